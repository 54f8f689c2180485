// results.cpp -- factor-file writer (src/factoring_results.hpp:507-525),
// excess-factor report (src/factors_buffer.hpp:172-192), checkpoint v1 codec
// (src/checkpoint.cpp:172-225) and the --print / --print-expression values
// (src/main.cpp:26-50) over a small non-negative big integer.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <sstream>

#include "cli.hpp"

namespace ctdcli {

// ------------------------------------------------------------- results
void write_results(std::ostream &out, factors_buffer &buf)
{
    const uint32_t m = buf.max_factors;
    std::string line;
    for (uint64_t i = 0; i < buf.numbers_count(); ++i) {
        uint64_t *f = buf.factors.data() + i * m;
        const uint32_t c = std::min(buf.counts[i], m);
        std::sort(f, f + c);
        line.clear();
        line += std::to_string(buf.n0 + i);
        line += " - ";
        for (uint32_t j = 0; j < c; ++j) {
            if (j)
                line += ", ";
            line += std::to_string(f[j]);
        }
        line += '\n';
        out << line;
    }
}

uint32_t max_factors_count(factors_buffer const &buf)
{
    return buf.counts.empty() ? 0 : *std::max_element(buf.counts.begin(), buf.counts.end());
}

uint64_t factors_count(factors_buffer const &buf)
{
    uint64_t s = 0;
    for (auto c : buf.counts)
        s += c;
    return s;
}

void report_excess_factors_if_any(factors_buffer const &buf, uint32_t &last_reported, std::ostream &log)
{
    const uint32_t mx = max_factors_count(buf);
    if (mx <= buf.max_factors || mx <= last_reported)
        return;
    last_reported = mx;
    const uint32_t suggested = ((mx / 64) + 1) * 64 + 64;
    log << "At least one number has factors count " << mx << " which exceeds the current storage limit ("
        << buf.max_factors << ").\n"
        << "Trial factoring continues normally, but some factors may be omitted from the recorded factor list "
           "for those terms.\nConsider restarting with\n  --max-factors-per-number "
        << suggested << std::endl;
}

// ----------------------------------------------------------- checkpoint
namespace {

constexpr uint32_t CHECKPOINT_FILE_VERSION = 1;

template <typename T>
void put(std::ostream &o, T const &v)
{
    o.write(reinterpret_cast<char const *>(&v), sizeof(v));
}

void put_str(std::ostream &o, std::string const &s)
{
    put(o, (size_t)s.size());
    o.write(s.data(), (std::streamsize)s.size());
}

template <typename T>
T get(std::istream &in, std::string const &path)
{
    T v{};
    if (!in.read(reinterpret_cast<char *>(&v), sizeof(v)))
        throw std::runtime_error{"Truncated checkpoint file `" + path + "'"};
    return v;
}

std::string get_str(std::istream &in, std::string const &path)
{
    auto n = get<size_t>(in, path);
    if (n > (size_t{1} << 32))
        throw std::runtime_error{"Corrupt checkpoint file `" + path + "'"};
    std::string s(n, '\0');
    if (n && !in.read(s.data(), (std::streamsize)n))
        throw std::runtime_error{"Truncated checkpoint file `" + path + "'"};
    return s;
}

}  // namespace

void write_checkpoint(std::string const &path, num_seq_spec const &spec, trial_factoring_options const &opts,
                      uint64_t last_processed_prime, factors_buffer const &buf)
{
    auto ns = std::chrono::duration_cast<std::chrono::nanoseconds>(
                  std::chrono::system_clock::now().time_since_epoch()).count();
    std::string tmp = path + ".tmp_" + std::to_string(ns);
    {
        std::ofstream out{tmp, std::ios::binary};
        if (!out)
            throw std::runtime_error{"Could not create temporary file `" + tmp + "'"};
        put(out, CHECKPOINT_FILE_VERSION);
        put(out, (uint32_t)spec.seq_id);
        put_str(out, spec.seq_params);
        put(out, opts.n0);
        put(out, opts.n1);
        put(out, opts.f0);
        put(out, opts.f1);
        put_str(out, opts.output_path.value_or(std::string{}));
        put(out, opts.max_factors_per_number);
        put(out, last_processed_prime);
        put(out, (uint64_t)buf.numbers_count());
        put(out, buf.max_factors);
        put(out, buf.n0);
        for (uint64_t i = 0; i < buf.numbers_count(); ++i) {
            put(out, buf.counts[i]);
            const uint32_t c = std::min(buf.counts[i], buf.max_factors);
            out.write(reinterpret_cast<char const *>(buf.factors.data() + i * buf.max_factors),
                      (std::streamsize)(c * sizeof(uint64_t)));
        }
        out.flush();
        if (!out)
            throw std::runtime_error{"Could not write checkpoint file `" + tmp + "'"};
    }
    std::filesystem::rename(tmp, path);
}

std::optional<checkpoint_data> load_checkpoint(std::string const &path)
{
    std::ifstream in{path, std::ios::binary};
    if (!in)
        return {};
    auto version = get<uint32_t>(in, path);
    if (version != CHECKPOINT_FILE_VERSION)
        throw std::runtime_error{"Unexpected version number `" + std::to_string(version) +
                                 "' found in checkpoint file"};
    checkpoint_data d;
    d.spec.seq_id = (num_seq_id)get<uint32_t>(in, path);
    d.spec.seq_params = get_str(in, path);
    auto &t = d.tf_options;
    t.n0 = get<uint64_t>(in, path);
    t.n1 = get<uint64_t>(in, path);
    t.f0 = get<uint64_t>(in, path);
    t.f1 = get<uint64_t>(in, path);
    auto op = get_str(in, path);
    if (!op.empty())
        t.output_path = op;
    t.max_factors_per_number = get<uint32_t>(in, path);
    d.last_processed_prime = get<uint64_t>(in, path);
    const auto numbers = get<uint64_t>(in, path);
    const auto m = get<uint32_t>(in, path);
    const auto n0 = get<uint64_t>(in, path);
    if (m == 0 || numbers > (uint64_t{1} << 40) / m)
        throw std::runtime_error{"Corrupt checkpoint file `" + path + "'"};
    d.buffer = factors_buffer{n0, numbers, m};
    for (uint64_t i = 0; i < numbers; ++i) {
        d.buffer.counts[i] = get<uint32_t>(in, path);
        const uint32_t c = std::min(d.buffer.counts[i], m);
        for (uint32_t j = 0; j < c; ++j)
            d.buffer.factors[i * m + j] = get<uint64_t>(in, path);
    }
    return d;
}

// --------------------------------------------------------------- bignum
namespace {

// non-negative integer, little-endian 64-bit limbs
struct Big {
    std::vector<uint64_t> l;
    Big() = default;
    explicit Big(uint64_t v)
    {
        if (v)
            l.push_back(v);
    }
    bool zero() const { return l.empty(); }
    void mul_small(uint64_t m)
    {
        unsigned __int128 c = 0;
        for (auto &x : l) {
            c += (unsigned __int128)x * m;
            x = (uint64_t)c;
            c >>= 64;
        }
        if (c)
            l.push_back((uint64_t)c);
        trim();
    }
    void add_small(uint64_t a)
    {
        for (size_t i = 0; a && i < l.size(); ++i) {
            l[i] += a;
            a = l[i] < a;
        }
        if (a)
            l.push_back(a);
    }
    void sub_small(uint64_t a)  // requires *this >= a
    {
        for (size_t i = 0; a && i < l.size(); ++i) {
            uint64_t o = l[i];
            l[i] -= a;
            a = l[i] > o;
        }
        trim();
    }
    void add(Big const &b)
    {
        if (b.l.size() > l.size())
            l.resize(b.l.size(), 0);
        uint64_t c = 0;
        for (size_t i = 0; i < l.size(); ++i) {
            unsigned __int128 s = (unsigned __int128)l[i] + (i < b.l.size() ? b.l[i] : 0) + c;
            l[i] = (uint64_t)s;
            c = (uint64_t)(s >> 64);
        }
        if (c)
            l.push_back(c);
    }
    void shl(uint64_t bits)
    {
        if (zero())
            return;
        const uint64_t w = bits / 64, b = bits % 64;
        std::vector<uint64_t> r(l.size() + w + 1, 0);
        for (size_t i = 0; i < l.size(); ++i) {
            r[i + w] |= l[i] << b;
            if (b)
                r[i + w + 1] |= l[i] >> (64 - b);
        }
        l.swap(r);
        trim();
    }
    void trim()
    {
        while (!l.empty() && !l.back())
            l.pop_back();
    }
    std::string str() const
    {
        if (zero())
            return "0";
        std::vector<uint64_t> t = l;
        std::vector<uint64_t> chunks;  // base 10^19
        const uint64_t B = 10000000000000000000ull;
        while (!t.empty()) {
            unsigned __int128 r = 0;
            for (size_t i = t.size(); i-- > 0;) {
                unsigned __int128 cur = (r << 64) | t[i];
                t[i] = (uint64_t)(cur / B);
                r = cur % B;
            }
            chunks.push_back((uint64_t)r);
            while (!t.empty() && !t.back())
                t.pop_back();
        }
        std::string s = std::to_string(chunks.back());
        char buf[32];
        for (size_t i = chunks.size() - 1; i-- > 0;) {
            std::snprintf(buf, sizeof buf, "%019llu", (unsigned long long)chunks[i]);
            s += buf;
        }
        return s;
    }
};

Big pow_big(uint64_t b, uint64_t e)
{
    Big r(1);
    for (uint64_t i = 0; i < e; ++i)
        r.mul_small(b);
    return r;
}

uint64_t digits(uint64_t b, uint64_t m)
{
    uint64_t d = 1;
    while (m /= b)
        ++d;
    return d;
}

// Sm_b(n), the concatenation of 1..n in base b
Big smarandache_value(uint64_t b, uint64_t n)
{
    Big v;
    for (uint64_t i = 1; i <= n; ++i) {
        uint64_t d = digits(b, i);
        uint64_t m = 1;
        for (uint64_t k = 0; k < d; ++k)
            m *= b;
        v.mul_small(m);
        v.add_small(i);
    }
    return v;
}

// smarandache.hpp:309-315 logb: floor(log_b(n))
uint64_t logb(uint64_t b, uint64_t n)
{
    uint64_t r = 0;
    while (n /= b)
        ++r;
    return r;
}

bool has_non_digit(std::string const &s)
{
    return std::any_of(s.begin(), s.end(), [](char c) { return c < '0' || c > '9'; });
}

// the expression for C_k, the constant of the closed form of Sm_b on digit
// class k (smarandache.cpp:264-288 describes its recursion)
std::string c_k_expression(uint64_t b, uint64_t k)
{
    const std::string bs = std::to_string(b);
    std::string c = bs;  // C_0 = b
    for (uint64_t i = 1; i <= k; ++i) {
        std::string b_i = (i != 1) ? bs + "^" + std::to_string(i) : bs;
        std::string b_i1 = bs + "^" + std::to_string(i + 1);
        std::string b_2i1 = bs + "^" + std::to_string(2 * i + 1);
        Big ex = pow_big(b, i - 1);
        ex.mul_small((b - 1));
        ex.mul_small(i);
        std::string pred = has_non_digit(c) ? "(" + c + ")" : c;
        c = "(" + pred + "*" + bs + "^" + ex.str() + " - (" + b_i + " - 1)^2 - " + b_i + ")/(" + b_i +
            " - 1)^2*(" + b_i1 + " - 1)^2 + " + b_2i1 + " - " + b_i + " + 1";
    }
    return c;
}

}  // namespace

int print_value(num_seq_spec const &spec, uint64_t n, std::ostream &out)
{
    uint32_t fam;
    uint64_t param;
    dispatch(spec, fam, param);
    construct_check(spec, param);
    Big v;
    bool negative = false;
    switch (spec.seq_id) {
    case num_seq_id::mersenne:
        v = Big(1);
        v.shl(n);
        v.sub_small(1);
        break;
    case num_seq_id::proth:
    case num_seq_id::riesel:
        v = Big(param);
        v.shl(n);
        if (spec.seq_id == num_seq_id::proth)
            v.add_small(1);
        else
            v.sub_small(1);
        break;
    case num_seq_id::proth_fixed_n:
    case num_seq_id::riesel_fixed_n:
        v = Big(n);
        v.shl(param);
        if (spec.seq_id == num_seq_id::proth_fixed_n)
            v.add_small(1);
        else if (v.zero())
            negative = true, v = Big(1);  // 0*2^n - 1 = -1
        else
            v.sub_small(1);
        break;
    case num_seq_id::smarandache: v = smarandache_value(param, n); break;
    case num_seq_id::fibonacci:
    case num_seq_id::lucas: {
        Big a(spec.seq_id == num_seq_id::fibonacci ? 0 : 2), b(1);
        for (uint64_t i = 0; i < n; ++i) {
            Big c = a;
            c.add(b);
            a = b;
            b = c;
        }
        v = a;
        break;
    }
    case num_seq_id::tribonacci: {
        Big a, b, c(1);
        for (uint64_t i = 0; i < n; ++i) {
            Big d = a;
            d.add(b);
            d.add(c);
            a = b;
            b = c;
            c = d;
        }
        v = a;
        break;
    }
    }
    out << (negative ? "-" : "") << v.str() << std::endl;
    return 0;
}

int print_expression(num_seq_spec const &spec, uint64_t n, std::ostream &out)
{
    uint32_t fam;
    uint64_t param;
    dispatch(spec, fam, param);
    construct_check(spec, param);
    switch (spec.seq_id) {
    case num_seq_id::mersenne: out << "2^" << n << "-1"; break;
    case num_seq_id::proth: out << param << "*2^" << n << " + 1"; break;
    case num_seq_id::riesel: out << param << "*2^" << n << " - 1"; break;
    case num_seq_id::proth_fixed_n: out << n << "*2^" << param << "+1"; break;
    case num_seq_id::riesel_fixed_n: out << n << "*2^" << param << "-1"; break;
    case num_seq_id::smarandache: {
        if (n < 2) {
            out << n;
            break;
        }
        const uint64_t b = param, k = logb(b, n);
        std::string ck = c_k_expression(b, k);
        if (has_non_digit(ck))
            ck = "(" + ck + ")";
        const std::string bk1 = k == 0 ? std::to_string(b) : std::to_string(b) + "^" + std::to_string(k + 1);
        // the exponent (k + 1)(n - b^k + 1), where b^k <= n
        uint64_t bk = 1;
        for (uint64_t i = 0; i < k; ++i)
            bk *= b;
        Big ex(n - bk + 1);
        ex.mul_small(k + 1);
        out << "(" << ck << "*" << b << "^" << ex.str() << " - (" << bk1 << " - 1)*" << n << " - " << bk1 << ")/("
            << bk1 << " - 1)^2";
        break;
    }
    default: out << "Expression not available"; break;
    }
    out << std::endl;
    return 0;
}

}  // namespace ctdcli
