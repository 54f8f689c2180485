// command_line.cpp -- the reference's command line (src/command_line.cpp:223-373)
// and help text (:391-603), restated: same flags, order rules and messages.
#include <cstring>
#include <sstream>
#include <unordered_map>

#include "cli.hpp"

namespace ctdcli {

num_seq_id num_seq_id_from_string(std::string const &s)
{
    static const std::unordered_map<std::string, num_seq_id> m{
        {"mersenne", num_seq_id::mersenne},       {"proth", num_seq_id::proth},
        {"riesel", num_seq_id::riesel},           {"smarandache", num_seq_id::smarandache},
        {"fibonacci", num_seq_id::fibonacci},     {"lucas", num_seq_id::lucas},
        {"proth_fixed_n", num_seq_id::proth_fixed_n}, {"riesel_fixed_n", num_seq_id::riesel_fixed_n},
        {"tribonacci", num_seq_id::tribonacci}};
    auto it = m.find(s);
    if (it == m.end())
        throw std::runtime_error{"Invalid number sequence id `" + s + "'"};
    return it->second;
}

std::string to_string(num_seq_id id)
{
    switch (id) {
    case num_seq_id::mersenne: return "mersenne";
    case num_seq_id::proth: return "proth";
    case num_seq_id::riesel: return "riesel";
    case num_seq_id::smarandache: return "smarandache";
    case num_seq_id::fibonacci: return "fibonacci";
    case num_seq_id::lucas: return "lucas";
    case num_seq_id::proth_fixed_n: return "proth_fixed_n";
    case num_seq_id::riesel_fixed_n: return "riesel_fixed_n";
    case num_seq_id::tribonacci: return "tribonacci";
    }
    return "<unknown number sequence id>";
}

namespace {

// std::from_chars on an unsigned 64-bit integer: leading digits, no sign
std::optional<uint64_t> parse_u64(std::string const &s)
{
    if (s.empty() || s[0] < '0' || s[0] > '9')
        return {};
    unsigned __int128 v = 0;
    for (char c : s) {
        if (c < '0' || c > '9')
            break;
        v = v * 10 + (c - '0');
        if (v >> 64)
            return {};
    }
    return (uint64_t)v;
}

}  // namespace

void dispatch(num_seq_spec const &spec, uint32_t &family, uint64_t &param)
{
    family = (uint32_t)spec.seq_id;
    param = 0;
    switch (spec.seq_id) {
    case num_seq_id::mersenne:
    case num_seq_id::fibonacci:
    case num_seq_id::lucas:
    case num_seq_id::tribonacci: return;
    case num_seq_id::proth:
    case num_seq_id::riesel: {
        bool proth = spec.seq_id == num_seq_id::proth;
        auto k = parse_u64(spec.seq_params);
        if (!k)
            throw std::runtime_error{"Missing or invalid k value `" + spec.seq_params + "' in " +
                                     (proth ? "Proth number" : "Riesel sequence") + " spec"};
        param = *k;
        return;
    }
    case num_seq_id::smarandache: {
        auto b = spec.seq_params.empty() ? std::optional<uint64_t>{10} : parse_u64(spec.seq_params);
        if (!b)
            throw std::runtime_error{"Invalid base `" + spec.seq_params + "' for Smarandache numbers"};
        if (*b < 2 || *b > 64)
            throw std::runtime_error{"Base `" + std::to_string(*b) + "' is not supported for Smarandache numbers"};
        param = *b;
        return;
    }
    case num_seq_id::proth_fixed_n:
    case num_seq_id::riesel_fixed_n: {
        bool proth = spec.seq_id == num_seq_id::proth_fixed_n;
        auto n = parse_u64(spec.seq_params);
        if (!n)
            throw std::runtime_error{"Missing or invalid n value `" + spec.seq_params + "' in " +
                                     (proth ? "Proth number" : "Riesel sequence") + " spec"};
        param = *n;
        return;
    }
    }
    throw std::runtime_error{"Unexpected number sequence id: " + std::to_string((int)spec.seq_id)};
}

void construct_check(num_seq_spec const &spec, uint64_t param)
{
    switch (spec.seq_id) {
    case num_seq_id::proth:
    case num_seq_id::riesel:
        if (!param)
            throw std::invalid_argument{std::string{spec.seq_id == num_seq_id::proth ? "Proth" : "Riesel"} +
                                        " parameter k must be non-zero"};
        break;
    case num_seq_id::proth_fixed_n:
    case num_seq_id::riesel_fixed_n:
        if (!param)
            throw std::invalid_argument{"Invalid n value zero for Riesel/Proth fixed n"};
        break;
    default: break;
    }
}

namespace {

using ex = command_line_parse_exception;

// value parsing as `std::istringstream{arg} >> val` (src/command_line.cpp:23-36)
template <typename T>
T read_value(char const *s)
{
    T v{};
    std::istringstream{s} >> v;
    return v;
}

template <>
uint16_t read_value<uint16_t>(char const *s)
{
    unsigned v = 0;
    std::istringstream{s} >> v;
    return (uint16_t)v;
}

template <typename T, typename Act>
bool eat_valued_option(char const *flag, char **&argv, Act act)
{
    if (!*argv || std::strcmp(*argv, flag))
        return false;
    ++argv;
    if (!*argv)
        throw ex{std::string{"Missing value for option "} + flag};
    if constexpr (std::is_same_v<T, std::string>)
        act(std::string{*argv});
    else
        act(read_value<T>(*argv));
    return true;
}

template <typename T, typename Dest>
bool parse_valued_option(char const *flag, Dest &dest, char **&argv)
{
    return eat_valued_option<T>(flag, argv, [&](T v) { dest = v; });
}

bool parse_no_progress(command_line_options &o, char **&argv)
{
    if (!std::strcmp(*argv, "--no-progress")) {
        o.is_progress_enabled = false;
        return true;
    }
    return false;
}

bool parse_verbosity(command_line_options &o, char **&argv)
{
    return eat_valued_option<uint16_t>("--verbosity", argv, [&](uint16_t v) {
        if (v > 4)
            throw ex{"Invalid value for option --verbosity"};
        o.verbosity_level = v;
    });
}

bool parse_segment_length(command_line_options &o, char **&argv)
{
    if (eat_valued_option<uint64_t>("--segment-length", argv, [&](uint64_t v) {
            if (o.segment_length)
                throw ex{"Invalid command line, --segment-length is not allowed when --segment-bits is present"};
            o.segment_length = v;
        }))
        return true;
    return eat_valued_option<int32_t>("--segment-bits", argv, [&](int32_t bits) {
        if (o.segment_length)
            throw ex{"Invalid command line, --segment-bits is not allowed when --segment-length is present"};
        if (bits < 0 || bits >= 64)
            throw ex{"value of option --segment-bits must be an integer in range [0, 63]"};
        o.segment_length = uint64_t{1} << bits;
    });
}

bool parse_device_options(command_line_options &o, char **&argv)
{
    return parse_valued_option<int32_t>("--device", o.device_id, argv) ||
           parse_valued_option<int32_t>("--grid-size", o.grid_size, argv) ||
           parse_valued_option<int32_t>("--block-size", o.block_size, argv);
}

void parse_num_seq(command_line_options &o, char **&argv)
{
    if (!eat_valued_option<std::string>("--num-seq", argv, [&](std::string spec) {
            try {
                auto comma = spec.find(',');
                if (comma != std::string::npos) {
                    o.seq_id = num_seq_id_from_string(spec.substr(0, comma));
                    o.seq_params = spec.substr(comma + 1);
                    if (o.seq_params.empty())
                        throw ex{"Invalid value for option --num-seq"};
                } else {
                    o.seq_id = num_seq_id_from_string(spec);
                }
            } catch (std::exception const &e) {
                throw ex{e.what()};
            }
            ++argv;
        }))
        throw ex{"Invalid command line, option --num-seq must come first"};
}

// resume mode (src/command_line.cpp:166-209)
void parse_resume(command_line_options &o, char **&argv)
{
    o.is_resuming = false;
    bool have_period = false;
    for (; *argv; ++argv) {
        if (eat_valued_option<std::string>("--resume", argv, [&](std::string p) {
                o.is_resuming = true;
                o.checkpoint_path = p;
            }))
            continue;
        if (parse_device_options(o, argv))
            continue;
        if (eat_valued_option<uint32_t>("--checkpoint-period", argv, [&](uint32_t v) {
                o.checkpoint_period = v;
                have_period = true;
            }))
            continue;
        if (parse_verbosity(o, argv))
            continue;
        if (parse_valued_option<uint32_t>("--threads", o.threads_count, argv))
            continue;
        if (parse_no_progress(o, argv))
            continue;
        if (parse_segment_length(o, argv))
            continue;
        if (!o.is_resuming && !have_period)
            return;
    }
    if (have_period && !o.is_resuming)
        throw ex{"Invalid command line, option --checkpoint-period is unexpected"};
}

}  // namespace

command_line_parser::command_line_parser(int argc, char **argv)
{
    if (argc == 1) {
        wants_usage_ = true;
        return;
    }
    if (argc == 2) {
        if (!std::strcmp(argv[1], "-h") || !std::strcmp(argv[1], "--help")) {
            wants_help_ = true;
            return;
        }
        if (!std::strcmp(argv[1], "--version")) {
            wants_version_ = true;
            return;
        }
        if (!std::strcmp(argv[1], "--autotest")) {
            wants_autotests_ = true;
            return;
        }
    }
    char **pp = argv + 1;
    options_ = command_line_options{};
    auto &o = *options_;
    parse_resume(o, pp);
    if (o.is_resuming)
        return;
    if (parse_verbosity(o, pp))
        ++pp;
    parse_num_seq(o, pp);

    trial_factoring_options tf{};
    bool have_start{}, have_end{}, have_bits{}, have_tf_start{}, have_tf_end{};
    for (; *pp; ++pp) {
        if (parse_verbosity(o, pp))
            continue;
        if (parse_valued_option<uint32_t>("--threads", o.threads_count, pp))
            continue;
        if (eat_valued_option<uint64_t>("--print", pp, [&](uint64_t n) {
                o.wants_value = true;
                o.n = n;
            }))
            return;
        if (eat_valued_option<uint64_t>("--print-expression", pp, [&](uint64_t n) {
                o.wants_expression = true;
                o.n = n;
            }))
            return;
        if (parse_device_options(o, pp))
            continue;
        if (parse_valued_option<uint64_t>("-s", tf.n0, pp)) {
            have_start = true;
            continue;
        }
        if (parse_valued_option<uint64_t>("-e", tf.n1, pp)) {
            have_end = true;
            continue;
        }
        if (eat_valued_option<uint16_t>("--tf-bits", pp, [&](uint16_t bits) {
                tf.f0 = 2;
                if (bits > 64)
                    throw ex{"The value of option --tf-bits must be an integer between 0 and 64"};
                tf.f1 = bits < 64 ? (uint64_t{1} << bits) : ~uint64_t{};
            })) {
            have_bits = true;
            continue;
        }
        if (parse_valued_option<uint64_t>("--tf-start", tf.f0, pp)) {
            have_tf_start = true;
            continue;
        }
        if (parse_valued_option<uint64_t>("--tf-end", tf.f1, pp)) {
            have_tf_end = true;
            continue;
        }
        if (have_bits && (have_tf_start || have_tf_end))
            throw ex{"Mixing --tf-bits with --tf-start and --tf-end is not allowed"};
        if (parse_no_progress(o, pp))
            continue;
        if (parse_valued_option<std::string>("--output", tf.output_path, pp))
            continue;
        if (parse_valued_option<uint32_t>("--checkpoint-period", o.checkpoint_period, pp))
            continue;
        if (parse_segment_length(o, pp))
            continue;
        if (parse_valued_option<uint32_t>("--max-factors-per-number", tf.max_factors_per_number, pp))
            continue;
    }
    if (!have_start || !(have_tf_start || have_bits) || !(have_tf_end || have_bits))
        throw ex{"Missing mandatory option"};
    if (!have_end)
        tf.n1 = tf.n0 + 1;
    if (tf.output_path && tf.output_path->empty())
        throw ex{"Invalid output path"};
    o.tf_options = tf;
}

void print_version(std::ostream &out)
{
    out << "cutrialdive version 1.2.0 (GB300 engine, libctd_gpu ABI " << ctd_abi_version() << ")" << std::endl
        << "[Compiled with gcc " << __VERSION__ << "] [device sieve] [sm_103a]" << std::endl;
}

static void print_usage_only(std::ostream &out)
{
    out << R"-(
  cutrialdive ( --version
              | ( -h | --help )
              | ( --num-seq <NUM_SEQ_ID>
                        ( --print n
                        | --print-expression n
                        | <trial factoring options>
                        )
                )
              | --resume <checkpoint_path> <resume options>
              )
              [<global options>]
)-";
}

void print_usage(std::ostream &out)
{
    print_usage_only(out);
    out << R"-(

  Type 'cutrialdive --help' for more.
)-";
}

void print_help(std::ostream &out)
{
    print_usage_only(out);
    out << R"-(

    --help
            prints this help and exits.
    --version
            prints the version number and exits.

    Global options
    --------------
    --threads <N>
            Accepted for compatibility; primes are sieved on the GPU.

    --verbosity <V>
            Set log verbosity level to V where V is an integer in range [0, 4]
            0: silent (no messages)
            1: normal
            2: verbose
            3: debug
            4: diagnostic

    Number sequence selection
    -------------------------
    --num-seq <NUM_SEQ_ID>
            Selects a number sequence to work on, possible values of
            <NUM_SEQ_ID> are: smarandache[,base], mersenne, proth,k,
            riesel,k, proth_fixed_n,n, riesel_fixed_n,n, fibonacci,
            lucas, tribonacci.
            smarandache,2 means Smarandache base 2, default is base 10.

    Print number
    ------------
    --print n
            prints S(n) in base 10.

    --print-expression n
            prints an expression whose evaluation yields S(n).

    Trial factoring
    ---------------
    If no output path is specified (i.e. option --output is missing) then
    the results are written to the console and checkpointing is deactivated.
    If an output path P is specified then P.chkpnt is reserved for the
    checkpoint file. The checkpoint file is deleted upon succesful completion
    of the trial factoring.

    -s n0   Processing will start with S(n0).
    -e n1   Processing will end with S(k), k the largest integer < n1.
            Default value is n0 + 1
    --tf-bits bits_count
            Use the primes in [2, 2^bits_count[.
    --tf-start f0
            Lower bound of the set of primes to consider.
    --tf-end f1
            Upper bound of the set of primes to consider (f1 is excluded).
    --no-progress
            Suppresses progress display.
    --output <path>
            Causes the output to be written to the given path.
    --checkpoint-period T
            Minimum duration in seconds between two checkpoint file savings.
    --segment-bits <L> | --segment-length <N>
            Length of a prime segment (unit of progress and checkpoints),
            default 2^26.
    --max-factors-per-number <N>
            Maximum number of factors stored per sequence term (default 32).

    --device <device_id>
            Id of the device to run the trial factoring on.
    --grid-size N
            Override default grid size (blocks per kernel launch) with N.
    --block-size N
            Override default block size (threads per block) with N.

    Resuming a trial factoring
    --------------------------
    --resume <checkpoint file path>
            Resume an interrupted trial factoring.
    The options available in resume mode are: --threads, --no-progress,
    --checkpoint-period, --device, --grid-size, --block-size, --segment-bits,
    --segment-length and the global options.
)-";
}

}  // namespace ctdcli
