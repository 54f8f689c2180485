// main.cpp -- the cutrialdive command-line drop-in (src/main.cpp:94-146)
// driving the GB300 engine through its C ABI.  Trial factoring follows the
// reference's trial_factor<Seq> (src/trial_factoring_impl.hpp:369-441) and
// trial_factor / resume_trial_factoring (src/trial_factoring.cpp:44-92):
// same status lines, output file, checkpoint file and exit codes.
#include <chrono>
#include <cmath>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <memory>

#include "cli.hpp"

namespace ctdcli {

namespace {

uint16_t g_verbosity = 1;

std::ostream &info(std::ostream &out)
{
    static std::ostream null{nullptr};
    return g_verbosity >= 1 ? out : null;
}

// progress line (src/progress.cpp:16-113)
class progress {
public:
    progress(uint64_t start, uint64_t target, uint32_t period_ms, std::ostream &out)
        : start_(start), target_(target), period_(period_ms), out_(out),
          width_(std::to_string(target).size()), t0_(std::chrono::steady_clock::now()), last_(t0_)
    {
    }
    void update(uint64_t current, uint64_t last_prime)
    {
        auto now = std::chrono::steady_clock::now();
        if (std::chrono::duration_cast<std::chrono::milliseconds>(now - last_).count() < period_ &&
            current != target_)
            return;
        const double pct = (double)(((unsigned __int128)(current - start_) * 10'000'000'000ull) /
                                    (target_ - start_)) / 100'000'000.0;
        const double el = std::chrono::duration<double>(now - t0_).count();
        out_ << "\r" << std::string(128, ' ') << "\r[" << std::setw(6) << std::fixed << std::setprecision(2) << pct
             << "% done][" << std::setw((int)width_) << last_prime << "][Elapsed ";
        duration(el);
        out_ << "]";
        if (current != target_ && pct > 0) {
            out_ << "[ETA ";
            duration((100 - pct) / pct * el);
            out_ << "]";
        }
        out_ << std::flush;
        last_ = std::chrono::steady_clock::now();
    }
    void end()
    {
        if (!ended_)
            out_ << std::endl;
        ended_ = true;
    }
    ~progress() { end(); }

private:
    void duration(double s)
    {
        if (s > 365 * 86400.0) {
            out_ << std::setw(8) << std::fixed << std::setprecision(2) << s / (365 * 86400) << " years";
            return;
        }
        if (s > 86400) {
            out_ << std::setw(3) << (int)(s / 86400) << "d ";
            s -= 86400 * (int)(s / 86400);
        }
        int h = (int)(s / 3600), m = (int)((s - 3600 * h) / 60), sec = (int)(s - 3600 * h - 60 * m);
        out_ << std::setw(2) << std::setfill('0') << h << ":" << std::setw(2) << m << ":" << std::setw(2) << sec
             << std::setfill(' ');
    }
    uint64_t start_, target_;
    uint32_t period_;
    std::ostream &out_;
    size_t width_;
    std::chrono::steady_clock::time_point t0_, last_;
    bool ended_{false};
};

struct run_state {
    num_seq_spec spec;
    trial_factoring_options opts;
    std::string checkpoint_path;  // empty: no checkpointing
    uint32_t checkpoint_period;
    factors_buffer *buf;
    progress *prog;
    std::chrono::steady_clock::time_point last_checkpoint;
    uint32_t excess_reported;
    std::ostream *out;
};

int on_progress(void *user, ctd_progress const *p, int snapshot)
{
    auto *st = static_cast<run_state *>(user);
    if (snapshot) {
        report_excess_factors_if_any(*st->buf, st->excess_reported, info(*st->out));
        write_checkpoint(st->checkpoint_path, st->spec, st->opts, p->last_prime, *st->buf);
        st->last_checkpoint = std::chrono::steady_clock::now();
        return CTD_CB_CONTINUE;
    }
    if (st->prog && p->last_prime)
        st->prog->update(p->segment_end, p->last_prime);
    if (!st->checkpoint_path.empty() && p->last_prime &&
        std::chrono::steady_clock::now() - st->last_checkpoint >= std::chrono::seconds(st->checkpoint_period))
        return CTD_CB_SNAPSHOT;
    return CTD_CB_CONTINUE;
}

struct engine {
    ctd_ctx *ctx{};
    explicit engine(int device)
    {
        int rc = ctd_open(device, &ctx);
        if (rc)
            throw std::runtime_error{std::string{"Error selecting device "} + std::to_string(device) + ": " +
                                     ctd_strerror(rc)};
    }
    ~engine() { ctd_close(ctx); }
};

void run(num_seq_spec const &spec, trial_factoring_options const &opts, tf_runtime_options const &rt,
         std::ostream &out, std::string const &checkpoint_path, checkpoint_data *resume)
{
    if (opts.n1 <= opts.n0) {
        out << "Range [" << opts.n0 << ", " << opts.n1 << "[ is empty, no number to process..." << std::endl;
        return;
    }
    if (opts.f1 <= opts.f0) {
        out << "Range [" << opts.f0 << ", " << opts.f1 << "[ is empty, no prime numbers to divide by..."
            << std::endl;
        return;
    }
    uint32_t family;
    uint64_t param;
    dispatch(spec, family, param);
    ctd_job job{family, opts.max_factors_per_number, param, opts.n0, opts.n1, opts.f0, opts.f1};

    std::unique_ptr<std::ofstream> file;
    if (opts.output_path) {
        file = std::make_unique<std::ofstream>(*opts.output_path);
        if (!*file)
            throw std::runtime_error{"Output: cannot open file " + *opts.output_path};
    }
    out << "Trial factoring starts, results will be written to "
        << (file ? "file `" + *opts.output_path + "'" : std::string{"the console."}) << std::endl;
    out << "TF range is [" << opts.f0 << ", " << opts.f1 << "[." << std::endl;
    if (!checkpoint_path.empty()) {
        out << "Checkpoint file will be written to `" << checkpoint_path << "' (period is " << rt.checkpoint_period
            << "s)." << std::endl;
        out << "Use `--resume " << std::quoted(checkpoint_path) << "' to resume execution." << std::endl;
    }
    construct_check(spec, param);
    if (ctd_check_job(&job))
        throw std::invalid_argument{"Invalid trial factoring job"};
    const auto t0 = std::chrono::steady_clock::now();
    engine eng{rt.device_id};
    {
        char name[256];
        uint64_t mem = 0;
        int sms = 0;
        ctd_device_info(eng.ctx, name, sizeof name, &mem, &sms);
        out << "Using GPU device " << rt.device_id << ": " << name << " (" << std::setprecision(3)
            << double(mem) / (1024.0 * 1024 * 1024) << " GiB)\n";
    }
    if (rt.grid_size || rt.block_size) {
        if (ctd_set_launch(eng.ctx, rt.grid_size.value_or(0), rt.block_size.value_or(0)))
            throw std::invalid_argument{"Invalid --grid-size / --block-size"};
    }
    factors_buffer buf;
    uint64_t resume_after = 0;
    if (resume) {
        buf = std::move(resume->buffer);
        resume_after = resume->last_processed_prime;
        if (buf.n0 != opts.n0 || buf.numbers_count() != opts.n1 - opts.n0 ||
            buf.max_factors != opts.max_factors_per_number)
            throw std::runtime_error{"Checkpoint factors buffer does not match its job"};
        out << "Resuming at the smallest prime > " << resume_after << "." << std::endl;
    } else {
        buf = factors_buffer{opts.n0, opts.n1 - opts.n0, opts.max_factors_per_number};
    }
    out << "Sieving for primes on the GPU." << std::endl;
    const uint64_t f0 = resume_after ? resume_after + 1 : opts.f0;
    std::unique_ptr<progress> prog;
    if (rt.is_progress_enabled && f0 < opts.f1)
        prog = std::make_unique<progress>(f0, opts.f1, rt.progress_period_ms, out);
    run_state st{spec, opts, checkpoint_path, rt.checkpoint_period, &buf, prog.get(),
                 std::chrono::steady_clock::now(), 0, &out};
    int rc = ctd_run_plain(eng.ctx, &job, buf.counts.data(), buf.factors.data(), resume_after, rt.segment_length,
                           on_progress, &st);
    if (prog)
        prog->end();
    if (rc)
        throw std::runtime_error{std::string{"Trial factoring failed: "} + ctd_last_error(eng.ctx)};
    report_excess_factors_if_any(buf, st.excess_reported, info(out));
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    out << "Trial factoring took " << secs << "s" << std::endl;
    write_results(file ? *file : out, buf);
    if (file) {
        file->flush();
        if (!*file)
            throw std::runtime_error{"Output: error writing " + *opts.output_path};
    }
    if (!checkpoint_path.empty())
        std::filesystem::remove(checkpoint_path);
    info(out) << "Maximum number of factors found for a single sequence term: " << max_factors_count(buf)
              << std::endl
              << "Overall number of factors found: " << factors_count(buf) << std::endl;
}

}  // namespace

void trial_factor(num_seq_spec const &spec, trial_factoring_options const &opts, tf_runtime_options const &rt,
                  std::ostream &out)
{
    std::string ck = opts.output_path ? *opts.output_path + ".chkpnt" : std::string{};
    run(spec, opts, rt, out, ck, nullptr);
}

void resume_trial_factoring(std::string const &checkpoint_path, tf_runtime_options const &rt, std::ostream &out)
{
    out << "Resuming from checkpoint `" << checkpoint_path << "'..." << std::endl;
    auto data = load_checkpoint(checkpoint_path);
    if (!data)
        throw std::runtime_error{"Failed to load checkpoint data from file `" + checkpoint_path + "'"};
    if (!data->tf_options.output_path)
        throw std::runtime_error{"Checkpoint without output path `" + checkpoint_path + "'"};
    std::string ck = *data->tf_options.output_path + ".chkpnt";
    run(data->spec, data->tf_options, rt, out, ck, &*data);
}

// --autotest: the reference's sieve known answers (src/autotests.cpp:136-351)
// run against the device sieve.  Like the reference, failures are printed and
// the exit status stays 0 (src/autotests.cpp:369).
int autotest(tf_runtime_options const &rt)
{
    struct kat {
        uint64_t lo, hi;
        std::vector<uint64_t> expected;
        long count;
    };
    const uint64_t s41 = (uint64_t(1) << 41) - (uint64_t(1) << 37) + (uint64_t(1) << 32);
    std::vector<kat> kats = {
        {256, 307, {257, 263, 269, 271, 277, 281, 283, 293}, -1},
        {1 << 16, (1 << 16) + 1, {}, 0},
        {1 << 16, (1 << 16) + 2, {65537}, 1},
        {(1ull << 31) - 1, (1ull << 31) + 100, {2147483647, 2147483659, 2147483693, 2147483713, 2147483743}, -1},
        {1, 1 << 17, {}, 12251},
        {1ull << 32, (1ull << 32) + 200,
         {4294967311ull, 4294967357ull, 4294967371ull, 4294967377ull, 4294967387ull, 4294967389ull, 4294967459ull,
          4294967477ull},
         8},
        {(1ull << 32) - 256, (1ull << 32) + 256, {}, 22},
        {65537ull * 65537 - 200, 65537ull * 65537 + 1,
         {4295098183, 4295098231, 4295098237, 4295098277, 4295098303, 4295098309, 4295098349}, 7},
        {(1ull << 34) - 200, (1ull << 34) + 200, {}, 11},
        {s41 - 1, s41 + 1000, {}, 26},
        {(1ull << 61) - 100, (1ull << 61), {2305843009213693907ull, 2305843009213693921ull, 2305843009213693951ull}, 3},
    };
    std::cout << "Executing self tests..." << std::endl;
    engine eng{rt.device_id};
    for (auto const &k : kats) {
        std::vector<uint64_t> primes(1 << 14);
        uint64_t n = 0;
        int rc = ctd_sieve(eng.ctx, k.lo, k.hi, primes.data(), primes.size(), &n);
        primes.resize(std::min<uint64_t>(n, primes.size()));
        bool ok = rc == 0 && (k.count < 0 || (long)n == k.count) && (k.expected.empty() || primes == k.expected);
        if (!ok)
            std::cerr << "Failure: sieve [" << k.lo << ", " << k.hi << ") gave " << n << " primes" << std::endl;
    }
    std::cout << "Done" << std::endl;
    return 0;
}

}  // namespace ctdcli

int main(int argc, char **argv)
{
    using namespace ctdcli;
    try {
        command_line_parser parser{argc, argv};
        if (parser.is_version_requested()) {
            print_version(std::cout);
            return 0;
        }
        if (parser.is_usage_requested()) {
            print_usage(std::cerr);
            return 1;
        }
        if (parser.is_help_requested()) {
            print_help(std::cout);
            return 0;
        }
        tf_runtime_options rt;
        if (parser.are_autotests_requested())
            return autotest(rt);
        auto const &o = *parser.get_options();
        if (o.threads_count)
            rt.threads_count = *o.threads_count;
        if (o.verbosity_level)
            rt.verbosity = *o.verbosity_level;
        g_verbosity = rt.verbosity;
        if (o.checkpoint_period)
            rt.checkpoint_period = *o.checkpoint_period;
        if (o.is_progress_enabled)
            rt.is_progress_enabled = *o.is_progress_enabled;
        if (o.segment_length)
            rt.segment_length = *o.segment_length;
        if (o.device_id)
            rt.device_id = *o.device_id;
        rt.grid_size = o.grid_size;
        rt.block_size = o.block_size;
        if (o.is_resuming) {
            resume_trial_factoring(*o.checkpoint_path, rt, std::cout);
            return 0;
        }
        num_seq_spec spec{o.seq_id, o.seq_params};
        if (o.wants_value)
            return print_value(spec, o.n, std::cout);
        if (o.wants_expression)
            return print_expression(spec, o.n, std::cout);
        trial_factor(spec, *o.tf_options, rt, std::cout);
    } catch (std::exception const &e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    return 0;
}
