// cli.hpp -- host side of the cutrialdive command-line drop-in.
//
// Same flags, messages, factor-file format and checkpoint layout as the
// reference CLI (src/command_line.cpp, src/main.cpp, src/trial_factoring.cpp,
// src/checkpoint.cpp, src/factoring_results.hpp); trial factoring itself goes
// through the C ABI of libctd_gpu.so (include/ctd_gpu.h).
#pragma once

#include <cstdint>
#include <optional>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ctd_gpu.h"

namespace ctdcli {

// src/num_seq_id.hpp:16-26
enum class num_seq_id : uint32_t {
    mersenne,
    proth,
    riesel,
    smarandache,
    fibonacci,
    lucas,
    proth_fixed_n,
    riesel_fixed_n,
    tribonacci
};

num_seq_id num_seq_id_from_string(std::string const &s);
std::string to_string(num_seq_id id);

struct num_seq_spec {
    num_seq_id seq_id{};
    std::string seq_params;
};

// (family, param) with the reference dispatch's parsing checks and messages
// (src/num_seq_dispatch.hpp:120-170)
void dispatch(num_seq_spec const &spec, uint32_t &family, uint64_t &param);
// the sequence constructors' checks (k != 0, n != 0: riesel_proth.hpp:133-141,
// riesel_proth_fixed_n.hpp:73-79), raised where the reference constructs the
// sequence (src/trial_factoring_impl.hpp:421)
void construct_check(num_seq_spec const &spec, uint64_t param);

// src/trial_factoring_options.hpp:15-31
struct trial_factoring_options {
    uint64_t n0{}, n1{}, f0{}, f1{};
    std::optional<std::string> output_path;
    uint32_t max_factors_per_number{32};
};

// src/trial_factoring_options.hpp:36-59 and src/options.hpp
struct tf_runtime_options {
    uint32_t threads_count{4};
    uint16_t verbosity{1};
    uint32_t checkpoint_period{360};
    uint32_t progress_period_ms{1000};
    bool is_progress_enabled{true};
    uint64_t segment_length{uint64_t{1} << 26};
    int32_t device_id{0};
    std::optional<int32_t> grid_size;
    std::optional<int32_t> block_size;
};

// src/command_line.hpp:26-58
struct command_line_options {
    bool is_resuming{};
    std::optional<std::string> checkpoint_path;
    std::optional<uint32_t> checkpoint_period;
    std::optional<bool> is_progress_enabled;
    std::optional<uint32_t> threads_count;
    std::optional<uint64_t> segment_length;
    std::optional<uint16_t> verbosity_level;
    std::optional<int32_t> device_id;
    std::optional<int32_t> grid_size;
    std::optional<int32_t> block_size;
    num_seq_id seq_id{};
    std::string seq_params;
    bool wants_value{};
    bool wants_expression{};
    uint64_t n{};
    std::optional<trial_factoring_options> tf_options;
};

class command_line_parse_exception : public std::runtime_error {
public:
    explicit command_line_parse_exception(std::string const &m) : std::runtime_error(m) {}
};

class command_line_parser {
public:
    command_line_parser(int argc, char **argv);
    bool is_help_requested() const { return wants_help_; }
    bool is_usage_requested() const { return wants_usage_; }
    bool is_version_requested() const { return wants_version_; }
    bool are_autotests_requested() const { return wants_autotests_; }
    std::optional<command_line_options> const &get_options() const { return options_; }

private:
    bool wants_help_{}, wants_usage_{}, wants_version_{}, wants_autotests_{};
    std::optional<command_line_options> options_;
};

void print_usage(std::ostream &out);
void print_help(std::ostream &out);
void print_version(std::ostream &out);

// ------------------------------------------------------------- results
// Host factors buffer in the reference layout (src/factors_buffer.hpp:77-86)
struct factors_buffer {
    uint64_t n0{};
    uint32_t max_factors{};
    std::vector<uint32_t> counts;
    std::vector<uint64_t> factors;
    factors_buffer() = default;
    factors_buffer(uint64_t n0_, uint64_t numbers, uint32_t maxf)
        : n0(n0_), max_factors(maxf), counts(numbers), factors(numbers * maxf) {}
    uint64_t numbers_count() const { return counts.size(); }
};

// '<n> - p1, p2' per term, factors sorted (src/factors_buffer.hpp:123-138,
// src/factoring_results.hpp:507-525)
void write_results(std::ostream &out, factors_buffer &buf);
uint32_t max_factors_count(factors_buffer const &buf);
uint64_t factors_count(factors_buffer const &buf);
// warning when a term found more factors than it can store
// (src/factors_buffer.hpp:172-192)
void report_excess_factors_if_any(factors_buffer const &buf, uint32_t &last_reported, std::ostream &log);

// ----------------------------------------------------------- checkpoint
// v1 layout of src/checkpoint.cpp:172-225 (native endian, LP64)
struct checkpoint_data {
    num_seq_spec spec;
    trial_factoring_options tf_options;
    uint64_t last_processed_prime{};
    factors_buffer buffer;
};

void write_checkpoint(std::string const &path, num_seq_spec const &spec, trial_factoring_options const &opts,
                      uint64_t last_processed_prime, factors_buffer const &buf);
std::optional<checkpoint_data> load_checkpoint(std::string const &path);

// ------------------------------------------------------------- values
// --print / --print-expression (src/main.cpp:26-50)
int print_value(num_seq_spec const &spec, uint64_t n, std::ostream &out);
int print_expression(num_seq_spec const &spec, uint64_t n, std::ostream &out);

// ------------------------------------------------------------- engine
void trial_factor(num_seq_spec const &spec, trial_factoring_options const &opts, tf_runtime_options const &rt,
                  std::ostream &out);
void resume_trial_factoring(std::string const &checkpoint_path, tf_runtime_options const &rt, std::ostream &out);
int autotest(tf_runtime_options const &rt);

}  // namespace ctdcli
