// deac_main.cpp -- the deac.e command line, a drop-in for the reference
// executable (src/deac/src/deac.cpp:1925-2197): the same flags and defaults,
// the same validation messages and exit codes, the same isf.bin input and
// .bin/.dat outputs.  The reconstruction itself runs on the GB300 through
// the C-ABI of include/deac_gb300.h; there is no CPU fallback.
//
// Compile-time variants of the reference are runtime flags here:
//   --model standard|hyperbolic|normalization   DEAC_MODEL
//   --zero_temperature                           ZeroT build type
//   --bosonic                                    one-sided genome (bdsf)
//   --allow_negative_spectral_weight             ALLOW_NEGATIVE_SPECTRAL_WEIGHT
//   --device N                                   CUDA device
//   --engine plain|split                         evaluation engine (same results)
//   --streams reference|counter                  draw layout (reference: its PRNG bit for bit)
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "deac_gb300.h"

namespace fs = std::filesystem;

namespace {

[[noreturn]] void fail_with_error(const std::string& msg) {
    std::cerr << msg << std::endl;
    std::exit(1);
}

struct Option {
    std::string short_name, long_name, help, default_text;
    bool is_flag = false;
};

const std::vector<Option>& options() {
    static const std::vector<Option> o = {
        {"-T", "--temperature", "Temperature of system.", "0", false},
        {"-N", "--number_of_generations", "Number of generations before genetic algorithm quits.", "100000", false},
        {"-P", "--population_size", "Size of initial population", "512", false},
        {"-M", "--genome_size", "Size of genome.", "512", false},
        {"", "--omega_max", "Maximum frequency to explore.", "60", false},
        {"", "--frequency_file", "Filename containing frequency partition (genome_size and omega_max will be ignored).", "", false},
        {"", "--normalize", "Normalize spectrum to the zeroeth moment.", "false", true},
        {"", "--use_negative_first_moment", "Calculate inverse first moment from ISF data and use it in fitness.", "false", true},
        {"", "--first_moment", "Set first frequency moment and use in fitness function.", "-1", false},
        {"", "--third_moment", "Set third frequency moment and use in fitness function.", "-1", false},
        {"", "--third_moment_error", "Set error for third frequency moment.", "0", false},
        {"-r", "--crossover_probability", "Initial probability for parent gene to become mutant vector gene.", "0.9", false},
        {"-u", "--self_adapting_crossover_probability", "Probability for `crossover_probability` to mutate.", "0.1", false},
        {"-F", "--differential_weight", "Initial weight factor when creating mutant vector.", "0.9", false},
        {"-v", "--self_adapting_differential_weight_probability", "Probability for `differential_weight` to mutate.", "0.1", false},
        {"-l", "--self_adapting_differential_weight_shift", "If `self_adapting_differential_weight_probability` mutate, new value is `l + m*rand()`.", "0.1", false},
        {"-m", "--self_adapting_differential_weight", "If `self_adapting_differential_weight_probability` mutate, new value is `l + m*rand()`.", "0.9", false},
        {"", "--stop_minimum_fitness", "Stopping criteria, if minimum fitness is below `stop_minimum_fitness` stop evolving.", "1", false},
        {"", "--seed", "Seed to pass to random number generator.", "0", false},
        {"", "--uuid", "UUID for run. If empty will be set to `seed`.", "", false},
        {"", "--number_of_seeds", "Reconstructions run together, with seeds seed, seed+1, ...; each writes its own files, named by its seed.", "1", false},
        {"", "--average_file", "File for the spectrum averaged over the seeds (float64, summed in the order of the seeds' names).", "", false},
        {"", "--save_state", "Save state of DEAC algorithm. Saves the random number generator, population, and population fitness.", "false", true},
        {"", "--save_directory", "Directory to save results in.", "./deacresults", false},
        {"", "--track_stats", "Track minimum fitness and other stats.", "false", true},
        {"", "--spectra_type", "Choose spectral type for kernel factors [spbsf, spfsf, bfull, ffull] (two-sided) or [bdsf] (with --bosonic).", "spfsf", false},
        {"", "--model", "Spectral model: standard, hyperbolic or normalization (the reference's DEAC_MODEL).", "standard", false},
        {"", "--zero_temperature", "Zero-temperature kernel exp(-tau*omega) (the reference's ZeroT build; needs --bosonic).", "false", true},
        {"", "--bosonic", "One-sided genome with the bosonic detailed-balance kernel (spectra_type bdsf).", "false", true},
        {"", "--allow_negative_spectral_weight", "Do not take the absolute value of mutant genes.", "false", true},
        {"", "--device", "CUDA device to run on.", "0", false},
        {"", "--engine", "Evaluation engine: plain (FP64 throughout) or split (tensor-core contraction with exact FP64 decisions; genome_size a multiple of 32).", "plain", false},
        {"", "--first_moment_formula", "First-moment fitness term: gpu ((m - m_i)/1.0)^2, the reference's GPU build, or cpu (m_i - m)^2/m, its CPU build.", "gpu", false},
        {"", "--streams", "Random draws: reference (the reference's per-gene generator states, its draws bit for bit) or counter (compact counter streams for large batches; both engines agree).", "reference", false},
    };
    return o;
}

void print_usage(std::ostream& os) {
    os << "Usage: deac-cpp [--help] [--version]";
    for (const auto& o : options()) os << " [" << o.long_name << (o.is_flag ? "" : " VAR") << "]";
    os << " isf_file\n\nPositional arguments:\n  isf_file\tbinary file containing isf data (tau, isf, error)\n\n"
       << "Optional arguments:\n  -h, --help\tshows help message and exits\n  --version\tprints version information and exits\n";
    for (const auto& o : options()) {
        os << "  ";
        if (!o.short_name.empty()) os << o.short_name << ", ";
        os << o.long_name << (o.is_flag ? "" : " VAR") << "\t" << o.help;
        if (!o.default_text.empty()) os << " [default: " << o.default_text << "]";
        os << "\n";
    }
}

struct Args {
    std::map<std::string, std::string> values;  // by long name
    std::vector<std::string> positional;
    bool has(const std::string& k) const { return values.count(k) != 0; }
};

// argparse-style parsing: "-X value", "--long value", "--long=value",
// flags without values, one positional argument.
bool parse(int argc, char** argv, Args& a, std::string& error) {
    std::map<std::string, const Option*> by_name;
    for (const auto& o : options()) {
        by_name[o.long_name] = &o;
        if (!o.short_name.empty()) by_name[o.short_name] = &o;
    }
    for (int k = 1; k < argc; ++k) {
        std::string tok = argv[k];
        if (tok == "-h" || tok == "--help") {
            print_usage(std::cout);
            std::exit(0);
        }
        if (tok == "--version") {
            std::cout << "2.0.0-rc1 (" << deac_version() << ")" << std::endl;
            std::exit(0);
        }
        std::string value;
        bool inline_value = false;
        if (tok.size() > 2 && tok.compare(0, 2, "--") == 0) {
            const size_t eq = tok.find('=');
            if (eq != std::string::npos) {
                value = tok.substr(eq + 1);
                tok = tok.substr(0, eq);
                inline_value = true;
            }
        }
        auto it = by_name.find(tok);
        if (it == by_name.end()) {
            // a lone "-" prefix that is not an option (e.g. "-1.0") is positional
            if (tok.size() > 1 && tok[0] == '-' && !std::isdigit((unsigned char)tok[1]) && tok[1] != '.') {
                error = "Unknown argument: " + tok;
                return false;
            }
            a.positional.push_back(tok);
            continue;
        }
        const Option& o = *it->second;
        if (o.is_flag) {
            a.values[o.long_name] = "1";
            continue;
        }
        if (!inline_value) {
            if (k + 1 >= argc) {
                error = o.long_name + ": expected 1 argument(s). 0 provided.";
                return false;
            }
            value = argv[++k];
        }
        a.values[o.long_name] = value;
    }
    if (a.positional.size() != 1) {
        error = a.positional.empty() ? "isf_file: 1 argument(s) expected. 0 provided."
                                     : "Maximum number of positional arguments exceeded";
        return false;
    }
    return true;
}

double get_double(const Args& a, const std::string& k, double def) {
    auto it = a.values.find(k);
    if (it == a.values.end()) return def;
    errno = 0;
    char* end = nullptr;
    const double v = std::strtod(it->second.c_str(), &end);
    if (end == it->second.c_str()) fail_with_error("invalid value for " + k + ": " + it->second);
    return v;
}

unsigned long get_ulong(const Args& a, const std::string& k, unsigned long def) {
    auto it = a.values.find(k);
    if (it == a.values.end()) return def;
    char* end = nullptr;
    const unsigned long v = std::strtoul(it->second.c_str(), &end, 10);
    if (end == it->second.c_str()) fail_with_error("invalid value for " + k + ": " + it->second);
    return v;
}

// raw little-endian float64 file (deac.cpp:58-100)
std::vector<double> load_doubles(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::fputs(("File error: " + path + "\n").c_str(), stderr);
        std::exit(1);
    }
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::rewind(f);
    if (size < 0 || size % (long)sizeof(double) != 0) {
        std::fclose(f);
        fail_with_error("File error: " + path + " does not contain a whole number of doubles");
    }
    const size_t n = (size_t)size / sizeof(double);
    if (n == 0) {
        std::fclose(f);
        fail_with_error("File error: " + path + " is empty");
    }
    std::vector<double> v(n);
    if (std::fread(v.data(), 1, (size_t)size, f) != (size_t)size) {
        std::fputs("Reading error", stderr);
        std::exit(3);
    }
    std::fclose(f);
    return v;
}

void write_array(const fs::path& p, const double* data, size_t n) {
    FILE* f = std::fopen(p.c_str(), "wb");
    if (!f) fail_with_error("File error: cannot write " + p.string());
    std::fwrite(data, sizeof(double), n, f);
    std::fclose(f);
}

const char* spectra_name(int st) {
    static const char* names[] = {"spbsf", "spfsf", "bfull", "ffull", "bdsf"};
    return names[st];
}

}  // namespace

int main(int argc, char** argv) {
    Args args;
    std::string perr;
    if (!parse(argc, argv, args, perr)) {
        std::cout << perr << std::endl;
        print_usage(std::cout);
        return 1;
    }

    deac_config cfg;
    deac_config_default(&cfg);
    cfg.bosonic = args.has("--bosonic") ? 1 : 0;
    cfg.zero_temperature = args.has("--zero_temperature") ? 1 : 0;
    cfg.allow_negative_weight = args.has("--allow_negative_spectral_weight") ? 1 : 0;
    const std::string model = args.has("--model") ? args.values.at("--model") : "standard";
    if (model == "standard") cfg.model = DEAC_MODEL_STANDARD;
    else if (model == "hyperbolic") cfg.model = DEAC_MODEL_HYPERBOLIC;
    else if (model == "normalization") cfg.model = DEAC_MODEL_NORMALIZATION;
    else {
        std::cout << "Please choose model from the following options: standard, hyperbolic, normalization" << std::endl;
        return 1;
    }

    const unsigned long seed_int = get_ulong(args, "--seed", 0);
    std::string uuid_str = args.has("--uuid") ? args.values.at("--uuid") : "";
    // several seeds in one batch replace the reference's one process per
    // seed (tools/generate_commands.sh:18-32); each seed's files keep the
    // single-run names, with the seed as the uuid
    const unsigned long n_seeds = get_ulong(args, "--number_of_seeds", 1);
    if (n_seeds < 1) fail_with_error("number_of_seeds must be at least 1");
    if (n_seeds > (1ul << 20)) fail_with_error("number_of_seeds must be at most 1048576");
    if (n_seeds > 1 && !uuid_str.empty())
        fail_with_error("uuid cannot be combined with number_of_seeds > 1: each seed's files are named by its seed");
    std::vector<unsigned long> seeds(n_seeds);
    std::vector<std::string> uuids(n_seeds);
    for (unsigned long k = 0; k < n_seeds; ++k) {
        seeds[k] = seed_int + k;
        uuids[k] = uuid_str.empty() ? std::to_string(seeds[k]) : uuid_str;
        std::cout << "uuid: " << uuids[k] << std::endl;
    }

    // spectra type (deac.cpp:2040-2058)
    const std::string spectra_type =
        args.has("--spectra_type") ? args.values.at("--spectra_type") : (cfg.bosonic ? "bdsf" : "spfsf");
    const std::vector<std::string> valid =
        cfg.bosonic ? std::vector<std::string>{"bdsf"} : std::vector<std::string>{"spbsf", "spfsf", "bfull", "ffull"};
    int st = -1;
    for (int k = 0; k < 5; ++k)
        if (spectra_type == spectra_name(k)) st = k;
    bool ok = false;
    for (const auto& v : valid) ok = ok || v == spectra_type;
    if (!ok) {
        std::cout << "Please choose spectra_type from the following options: "
                  << (cfg.bosonic ? "bdsf" : "spbsf, spfsf, bfull, ffull") << std::endl;
        return 1;
    }
    cfg.spectra_type = st;
    if (cfg.zero_temperature && !cfg.bosonic)
        fail_with_error("zero temperature requires the one-sided (bosonic) genome: add --bosonic");

    // ISF input (deac.cpp:2060-2087)
    const std::string isf_file = args.positional[0];
    std::vector<double> data = load_doubles(isf_file);
    if (data.size() % 3 != 0) fail_with_error("ISF input file must contain tau, isf, and error arrays of equal length");
    const size_t nt = data.size() / 3;
    if (nt < 2) fail_with_error("ISF input file must contain at least two timeslices");
    const double* tau = data.data();
    const double* isf = data.data() + nt;
    const double* err = data.data() + 2 * nt;
    for (size_t i = 0; i < nt; ++i) {
        if (!std::isfinite(tau[i]) || !std::isfinite(isf[i]) || !std::isfinite(err[i]))
            fail_with_error("ISF input file contains non-finite values");
        if (!cfg.bosonic && (st == DEAC_SPECTRA_SPBSF || st == DEAC_SPECTRA_SPFSF) && isf[i] > 0.0)
            fail_with_error("positive ISF values are not supported for single-particle spectra");
        if (err[i] <= 0.0) fail_with_error("ISF input errors must be positive");
    }

    cfg.seed = seed_int;
    cfg.temperature = get_double(args, "--temperature", 0.0);
    if (!cfg.zero_temperature && (!std::isfinite(cfg.temperature) || cfg.temperature <= 0.0))
        fail_with_error("temperature must be positive for non-ZeroT builds");
    cfg.number_of_generations = get_ulong(args, "--number_of_generations", 100000);
    cfg.population_size = get_ulong(args, "--population_size", 512);
    if (cfg.number_of_generations < 2) fail_with_error("number_of_generations must be at least 2");
    if (cfg.population_size < 4) fail_with_error("population_size must be at least 4");

    // frequency grid (deac.cpp:2108-2138)
    std::vector<double> frequency;
    if (args.has("--frequency_file")) {
        frequency = load_doubles(args.values.at("--frequency_file"));
    } else {
        const size_t m = get_ulong(args, "--genome_size", 512);
        const double omega_max = get_double(args, "--omega_max", 60.0);
        if (m < 2) fail_with_error("genome_size must be at least 2");
        if (!std::isfinite(omega_max) || omega_max <= 0.0) fail_with_error("omega_max must be positive");
        const double d = omega_max / (m - 1);
        frequency.resize(m);
        for (size_t i = 0; i < m; ++i) frequency[i] = i * d;
    }
    if (frequency.size() < 2) fail_with_error("frequency_file must contain at least two frequencies");
    for (size_t i = 0; i < frequency.size(); ++i) {
        if (!std::isfinite(frequency[i]) || frequency[i] < 0.0)
            fail_with_error("frequencies must be finite and non-negative");
        if (i > 0 && frequency[i] < frequency[i - 1]) fail_with_error("frequencies must be sorted in non-decreasing order");
    }

    cfg.normalize = args.has("--normalize") ? 1 : 0;
    cfg.use_negative_first_moment = args.has("--use_negative_first_moment") ? 1 : 0;
    cfg.first_moment = get_double(args, "--first_moment", -1.0);
    cfg.third_moment = get_double(args, "--third_moment", -1.0);
    cfg.third_moment_error = get_double(args, "--third_moment_error", 0.0);
    if (!std::isfinite(cfg.first_moment)) fail_with_error("first_moment must be finite");
    if (!std::isfinite(cfg.third_moment)) fail_with_error("third_moment must be finite");
    if (cfg.third_moment >= 0.0 && (!std::isfinite(cfg.third_moment_error) || cfg.third_moment_error <= 0.0))
        fail_with_error("third_moment_error must be positive when third_moment is used");
    cfg.crossover_probability = get_double(args, "--crossover_probability", 0.9);
    cfg.self_adapting_crossover_probability = get_double(args, "--self_adapting_crossover_probability", 0.1);
    cfg.differential_weight = get_double(args, "--differential_weight", 0.9);
    cfg.self_adapting_differential_weight_probability =
        get_double(args, "--self_adapting_differential_weight_probability", 0.1);
    cfg.self_adapting_differential_weight_shift = get_double(args, "--self_adapting_differential_weight_shift", 0.1);
    cfg.self_adapting_differential_weight = get_double(args, "--self_adapting_differential_weight", 0.9);
    cfg.stop_minimum_fitness = get_double(args, "--stop_minimum_fitness", 1.0);
    cfg.track_stats = args.has("--track_stats") ? 1 : 0;
    const int device = (int)get_ulong(args, "--device", 0);
    const std::string engine_name = args.has("--engine") ? args.values.at("--engine") : "plain";
    if (engine_name != "plain" && engine_name != "split") fail_with_error("--engine must be plain or split");
    const int32_t engine = engine_name == "split" ? DEAC_ENGINE_SPLIT_BF16 : DEAC_ENGINE_PLAIN_FP64;
    const std::string fm_name = args.has("--first_moment_formula") ? args.values.at("--first_moment_formula") : "gpu";
    if (fm_name != "gpu" && fm_name != "cpu") fail_with_error("--first_moment_formula must be gpu or cpu");
    cfg.first_moment_formula = fm_name == "cpu" ? DEAC_FIRST_MOMENT_CPU : DEAC_FIRST_MOMENT_GPU;
    const std::string streams_name = args.has("--streams") ? args.values.at("--streams") : "reference";
    if (streams_name != "reference" && streams_name != "counter")
        fail_with_error("--streams must be reference or counter");
    const int32_t streams = streams_name == "counter" ? DEAC_STREAMS_COUNTER : DEAC_STREAMS_REFERENCE;

    const fs::path save_directory(args.has("--save_directory") ? args.values.at("--save_directory") : "./deacresults");
    std::error_code ec;
    fs::create_directory(save_directory, ec);
    if (ec) fail_with_error("cannot create save_directory " + save_directory.string() + ": " + ec.message());

    const std::string prefix = (cfg.zero_temperature ? std::string("deac-zT") : std::string("deac-")) + spectra_type;
    auto log_filename = [&](unsigned long k) { return save_directory / (prefix + "_log_" + uuids[k] + ".dat"); };
    for (unsigned long k = 0; k < n_seeds; ++k) {
        std::ofstream log(log_filename(k), std::ios_base::out | std::ios_base::app);
        log << "uuid: " << uuids[k] << std::endl;
        log << "isf_file: " << isf_file << std::endl;
    }
    const std::string average_file = args.has("--average_file") ? args.values.at("--average_file") : "";
    if (!average_file.empty()) {
        const fs::path parent = fs::path(average_file).parent_path();
        if (!parent.empty() && !fs::is_directory(parent))
            fail_with_error("average_file directory does not exist: " + parent.string());
    }

    // inside deac(): zero temperature disables the negative first moment
    // (deac.cpp:234-239); the GPU path fixes the first-moment error to 1
    // (deac.cpp:622-627)
    if (cfg.zero_temperature) {
        if (cfg.use_negative_first_moment)
            std::cout << "use_negative_first_moment disabled for zero temperature build" << std::endl;
        cfg.use_negative_first_moment = 0;
        cfg.temperature = 0.0;
    }
    if (cfg.first_moment >= 0.0 && cfg.first_moment_formula == DEAC_FIRST_MOMENT_GPU)
        std::cout << "WARNING: setting first_moment_error to 1.0." << std::endl;

    deac_batch* batch = nullptr;
    int rc = deac_batch_create(device, nullptr, engine, &batch);
    if (rc == DEAC_OK) rc = deac_batch_set_streams(batch, streams);
    for (unsigned long k = 0; k < n_seeds && rc == DEAC_OK; ++k) {
        cfg.seed = seeds[k];
        rc = deac_batch_add_run(batch, &cfg, tau, isf, err, nt, frequency.data(), frequency.size(), nullptr);
    }
    if (rc == DEAC_OK) rc = deac_batch_run(batch);

    // the seeds' outputs in the order of their names, which is the order the
    // reference's averaging sums them in
    // (tools/plot_simple_average_deac_results.py:10-27)
    std::vector<unsigned long> order(n_seeds);
    for (unsigned long k = 0; k < n_seeds; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](unsigned long a, unsigned long b) { return uuids[a] < uuids[b]; });
    std::vector<double> average;
    std::vector<double> dsf, freq_out, s_mean, s_min, s_sq;
    static const char* build_names[] = {"USE_STANDARD_MODEL", "USE_HYPERBOLIC_MODEL", "USE_NORMALIZATION_MODEL"};
    for (unsigned long n = 0; n < n_seeds && rc == DEAC_OK; ++n) {
        const unsigned long k = order[n];
        deac_run_result res{};
        rc = deac_batch_result(batch, (uint32_t)k, &res);
        if (rc != DEAC_OK) break;
        dsf.resize(res.spectrum_length);
        freq_out.resize(res.spectrum_length);
        if (cfg.track_stats) {
            s_mean.resize(res.stats_length);
            s_min.resize(res.stats_length);
            s_sq.resize(res.stats_length);
        }
        rc = deac_batch_fetch(batch, (uint32_t)k, dsf.data(), freq_out.data(),
                              cfg.track_stats ? s_mean.data() : nullptr, cfg.track_stats ? s_min.data() : nullptr,
                              cfg.track_stats ? s_sq.data() : nullptr);
        if (rc != DEAC_OK) break;
        if (n == 0) {
            average = dsf;
        } else {
            for (size_t i = 0; i < average.size(); ++i) average[i] += dsf[i];
        }

        // outputs (deac.cpp:1687-1769)
        const std::string& uuid = uuids[k];
        const fs::path dsf_filename = save_directory / (prefix + "_dsf_" + uuid + ".bin");
        const fs::path frequency_filename = save_directory / (prefix + "_frequency_" + uuid + ".bin");
        write_array(dsf_filename, dsf.data(), dsf.size());
        write_array(frequency_filename, freq_out.data(), freq_out.size());
        fs::path mean_fn, min_fn, sq_fn;
        if (cfg.track_stats) {
            mean_fn = save_directory / (prefix + "_stats_fitness-mean_" + uuid + ".bin");
            min_fn = save_directory / (prefix + "_stats_fitness-minimum_" + uuid + ".bin");
            sq_fn = save_directory / (prefix + "_stats_fitness-squared-mean_" + uuid + ".bin");
            write_array(mean_fn, s_mean.data(), s_mean.size());
            write_array(min_fn, s_min.data(), s_min.size());
            write_array(sq_fn, s_sq.data(), s_sq.size());
        }

        std::ofstream log(log_filename(k), std::ios_base::out | std::ios_base::app);
        log << "build: " << build_names[cfg.model] << std::endl;
        log << "kernel: " << spectra_type << std::endl;
        log << "temperature: " << cfg.temperature << std::endl;
        log << "number_of_generations: " << cfg.number_of_generations << std::endl;
        log << "number_of_timeslices: " << nt << std::endl;
        log << "population_size: " << cfg.population_size << std::endl;
        log << "genome_size: " << frequency.size() << std::endl;
        log << "normalize: " << cfg.normalize << std::endl;
        log << "use_negative_first_moment: " << cfg.use_negative_first_moment << std::endl;
        log << "first_moment: " << cfg.first_moment << std::endl;
        log << "third_moment: " << cfg.third_moment << std::endl;
        log << "third_moment_error: " << cfg.third_moment_error << std::endl;
        log << "crossover_probability: " << cfg.crossover_probability << std::endl;
        log << "self_adapting_crossover_probability: " << cfg.self_adapting_crossover_probability << std::endl;
        log << "differential_weight: " << cfg.differential_weight << std::endl;
        log << "self_adapting_differential_weight_probability: " << cfg.self_adapting_differential_weight_probability
            << std::endl;
        log << "self_adapting_differential_weight_shift: " << cfg.self_adapting_differential_weight_shift << std::endl;
        log << "self_adapting_differential_weight: " << cfg.self_adapting_differential_weight << std::endl;
        log << "stop_minimum_fitness: " << cfg.stop_minimum_fitness << std::endl;
        log << "track_stats: " << cfg.track_stats << std::endl;
        log << "seed: " << seeds[k] << std::endl;
        log << "best_dsf_filename: " << dsf_filename << std::endl;
        log << "frequency_filename: " << frequency_filename << std::endl;
        log << "generation: " << res.generation << std::endl;
        std::cout << "generation: " << res.generation << std::endl;
        log << "minimum_fitness: " << res.minimum_fitness << std::endl;
        std::cout << "minimum_fitness: " << res.minimum_fitness << std::endl;
        if (cfg.track_stats) {
            log << "fitness_mean_filename: " << mean_fn << std::endl;
            log << "fitness_minimum_filename: " << min_fn << std::endl;
            log << "fitness_squared_mean_filename: " << sq_fn << std::endl;
        }
    }
    if (rc != DEAC_OK) {
        std::cerr << "deac-gb300: " << deac_last_error() << std::endl;
        deac_batch_destroy(batch);
        return 2;
    }
    deac_batch_destroy(batch);
    if (!average_file.empty()) {
        for (double& v : average) v /= (double)n_seeds;
        write_array(average_file, average.data(), average.size());
    }
    return 0;
}
