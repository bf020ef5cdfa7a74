// plbm_benchmark.cpp — the reference's benchmark driver (lbm::benchmark::Benchmark,
// src/lbm/benchmark/benchmark.cpp:30-383, include/lbm/benchmark/benchmark.hpp) on libplbm handlers.
//
//   phase 0  algorithms x dataLayouts x work-group sizes (+ lptl with "auto"), 10 steps each
//   phase 1  the same sweep for timeSteps; per algorithm the data layout and work-group size with the
//            lowest mean (initialisation + run) time are kept
//   phase 2  each algorithm's kept setup on every phaseTwoScenarios entry
//
// Each configuration runs testRunsPerConfig times; a run is handler creation (the reference's
// initialize(), timed as "initializationTimes") then start() + block_until_finished() (timed as
// "runtimes").  Output files, names and JSON shape are the reference's; every entry also lists
// "mlups" and, given the measured copy bandwidth, "hbmFraction" per run.
#include "../../include/plbm_c.h"
#include "plbm_json.hpp"
#include "plbm_power.h"

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

using plbm::Json;
namespace fs = std::filesystem;

// Benchmark::get_work_group_sizes (benchmark.cpp:30-62): per quarter of the maximum, the sizes
// region - 0..3 that are powers of 4 or 2, plus the first even and the first odd other size.
std::vector<unsigned> work_group_sizes(unsigned max_wg)
{
    std::vector<unsigned> out;
    for (unsigned i = 4; i >= 1; --i) {
        const unsigned region = i * max_wg / 4;
        bool even = false, odd = false;
        for (unsigned j = 0; j < 4; ++j) {
            const unsigned size = region - j;
            if (plbm::which_power_of_4(size) || plbm::which_power_of_2(size)) out.push_back(size);
            else if (!(size % 2) && !even) { out.push_back(size); even = true; }
            else if ((size % 2) && !odd) { out.push_back(size); odd = true; }
        }
    }
    return out;
}

// benchmark.cpp:18-28 and seconds_to_time_format (benchmark.hpp)
struct Progress {
    int total, done = 0;
    double avg = 0, remaining = 0;
    explicit Progress(int n) : total(n) {}
    void advance(double seconds)
    {
        ++done;
        avg = ((done - 1) * avg + seconds) / done;
        remaining = (total - done) * avg;
        unsigned s = (unsigned)remaining;
        const unsigned d = s / 86400; s -= d * 86400;
        const unsigned h = s / 3600; s -= h * 3600;
        const unsigned m = s / 60; s -= m * 60;
        std::printf("Progress: %d / %d (%d%%), remaining time estimation: %ud, %uh, %um, %us \n", done, total,
                    (int)std::floor(100.0 * done / total), d, h, m, s);
        std::fflush(stdout);
    }
};

Json jarr() { Json j; j.type = Json::ARRAY; return j; }
Json jobj() { Json j; j.type = Json::OBJECT; return j; }

class Bench {
  public:
    Bench(const plbm_properties &base, const plbm_options *opts, std::string out_root, std::string device,
          double hbm_gbs, unsigned runs)
        : out_(std::move(out_root)), device_(std::move(device)), hbm_(hbm_gbs), runs_(runs)
    {
        p_ = base;
        alg_ = base.algorithm; lay_ = base.data_layout;
        if (opts) opts_ = *opts;
        else plbm_default_options(&opts_);
        opts_.mask = nullptr;   // the benchmark runs the scenarios' own geometry
        bytes_node_ = 18.0 * (opts_.precision == PLBM_F32_REF || opts_.precision == PLBM_F32 ? 4
                              : opts_.precision == PLBM_F16S || opts_.precision == PLBM_BF16S ||
                                        opts_.precision == PLBM_F16C
                                    ? 2
                                    : 8);
    }

    // One run; false if the configuration was rejected (the error is printed).
    bool run_once(double &init_s, double &run_s)
    {
        plbm_properties q = p_;
        q.algorithm = alg_.c_str(); q.data_layout = lay_.c_str(); q.scenario = scn_.c_str();
        const auto t0 = std::chrono::steady_clock::now();
        plbm_handler *h = nullptr;
        int rc = plbm_create(&q, &opts_, &h);
        const auto t1 = std::chrono::steady_clock::now();
        if (rc == PLBM_OK) rc = plbm_start(h);
        if (rc == PLBM_OK) rc = plbm_block_until_finished(h);
        const auto t2 = std::chrono::steady_clock::now();
        if (rc != PLBM_OK) {
            std::printf("configuration %s/%s/wg %u/%s rejected: %s\n", alg_.c_str(), lay_.c_str(), q.work_group_size,
                        scn_.c_str(), plbm_last_error(h));
            if (h) plbm_destroy(h);
            return false;
        }
        plbm_destroy(h);
        init_s = std::chrono::duration<double>(t1 - t0).count();
        run_s = std::chrono::duration<double>(t2 - t1).count();
        return true;
    }

    static void push(Json &entry, const char *key, double v)
    {
        Json &a = entry.set(key);
        a.type = Json::ARRAY;
        a.arr.push_back(plbm::jnum(v, false));
    }

    void record(Json &entry, double init_s, double run_s)
    {
        push(entry, "initializationTimes", init_s);
        push(entry, "runtimes", run_s);
        const double nodes = (double)p_.vertical_nodes * p_.horizontal_nodes * p_.time_steps;
        push(entry, "mlups", nodes / run_s / 1e6);
        if (hbm_ > 0) push(entry, "hbmFraction", nodes * bytes_node_ / run_s / (hbm_ * 1e9));
    }

    Json file_header(const std::string &algorithm) const
    {
        Json f = jobj();
        f.set("device") = plbm::jstr(device_);
        f.set("algorithm") = plbm::jstr(algorithm);
        f.set("verticalNodes") = plbm::jnum(p_.vertical_nodes + 2, true);
        f.set("horizontalNodes") = plbm::jnum(p_.horizontal_nodes + 2, true);
        return f;
    }

    static Json empty_entry(Json wg)
    {
        Json e = jobj();
        e.set("workGroupSize") = std::move(wg);
        e.set("initializationTimes") = jarr();
        e.set("runtimes") = jarr();
        e.set("mlups") = jarr();
        return e;
    }

    void write(const fs::path &path, const Json &j)
    {
        std::string s;
        plbm::json_dump(s, j);
        std::ofstream(path) << s;
    }

    // phase_0_and_1_inner_loop (benchmark.cpp:137-193): every data layout at the current
    // algorithm and work-group size, testRunsPerConfig runs each.
    void inner_0_1(int phase, size_t index, const fs::path &file, Json &data, Progress &progress)
    {
        for (const auto &layout : layouts) {
            lay_ = layout;
            double total = 0;
            int ok = 0;
            for (unsigned r = 0; r < runs_; ++r) {
                const auto b0 = std::chrono::steady_clock::now();
                double is = 0, rs = 0;
                if (run_once(is, rs)) {
                    record(data.set(layout).arr[index], is, rs);
                    total += is + rs;
                    ++ok;
                }
                progress.advance(std::chrono::duration<double>(std::chrono::steady_clock::now() - b0).count());
                write(file, data);
            }
            if (phase == 1 && ok == (int)runs_) {
                const double avg = total / runs_;
                if (avg < best_time[alg_]) {
                    best_time[alg_] = avg;
                    best_layout[alg_] = layout;
                    best_wg[alg_] = p_.work_group_size;
                }
            }
        }
    }

    // phase_0_and_1_helper (benchmark.cpp:195-240)
    void phase_0_1(int phase)
    {
        std::printf("====================================================================================================\n"
                    "Starting benchmark phase %d.\n\n", phase);
        const fs::path dir = fs::path(out_) / "benchmarks" / ("phase" + std::to_string(phase));
        fs::create_directories(dir);
        int total = (int)(algorithms.size() * layouts.size() * wgs.size() * runs_);
        if (linear) total += (int)(layouts.size() * runs_);
        Progress progress(total);
        for (const auto &algorithm : algorithms) {
            alg_ = algorithm;
            const fs::path file = dir / ("results_phase" + std::to_string(phase) + "_" + algorithm + "_" + device_ + ".json");
            Json data = file_header(algorithm);
            for (const auto &layout : layouts) {
                Json list = jarr();
                for (unsigned wg : wgs) list.arr.push_back(empty_entry(plbm::jnum(wg, true)));
                data.set(layout) = std::move(list);
            }
            for (size_t j = 0; j < wgs.size(); ++j) {
                p_.work_group_size = wgs[j];
                inner_0_1(phase, j, file, data, progress);
            }
        }
        if (linear) {
            alg_ = "lptl";
            const fs::path file = dir / ("results_phase" + std::to_string(phase) + "_lptl_" + device_ + ".json");
            Json data = file_header("lptl");
            for (const auto &layout : layouts) {
                Json list = jarr();
                list.arr.push_back(empty_entry(plbm::jstr("auto")));
                data.set(layout) = std::move(list);
            }
            inner_0_1(phase, 0, file, data, progress);
        }
        std::printf("\nSuccessfully completed phase %d of benchmark\n"
                    "====================================================================================================\n\n", phase);
    }

    // phase_2 (benchmark.cpp:312-383)
    void phase_2()
    {
        std::printf("====================================================================================================\n"
                    "Starting benchmark phase 2.\n\n");
        const fs::path dir = fs::path(out_) / "benchmarks" / "phase2";
        fs::create_directories(dir);
        int total = (int)(algorithms.size() * scenarios.size() * runs_);
        if (linear) total += (int)(scenarios.size() * runs_);
        Progress progress(total);
        std::vector<std::string> algs = algorithms;
        if (linear) algs.push_back("lptl");
        for (const auto &algorithm : algs) {
            alg_ = algorithm;
            lay_ = best_layout[algorithm];
            p_.work_group_size = best_wg[algorithm];
            for (const auto &scenario : scenarios) {
                scn_ = scenario;
                const fs::path file = dir / ("phase2_" + algorithm + "_" + scenario + "_" + device_ + ".json");
                Json data = jobj();
                data.set("device") = plbm::jstr(device_);
                data.set("algorithm") = plbm::jstr(algorithm);
                data.set("dataLayout") = plbm::jstr(lay_);
                data.set("workGroupSize") = algorithm == "lptl" ? plbm::jstr("auto") : plbm::jnum(p_.work_group_size, true);
                data.set("verticalNodes") = plbm::jnum(p_.vertical_nodes + 2, true);
                data.set("horizontalNodes") = plbm::jnum(p_.horizontal_nodes + 2, true);
                data.set("scenario") = plbm::jstr(scenario);
                data.set("initializationTimes") = jarr();
                data.set("runtimes") = jarr();
                data.set("mlups") = jarr();
                for (unsigned r = 0; r < runs_; ++r) {
                    const auto b0 = std::chrono::steady_clock::now();
                    double is = 0, rs = 0;
                    if (run_once(is, rs)) record(data, is, rs);
                    progress.advance(std::chrono::duration<double>(std::chrono::steady_clock::now() - b0).count());
                    write(file, data);
                }
            }
        }
        scn_ = "Hagen-Poiseuille";
        std::printf("\nSuccessfully completed phase 2 of benchmark\n"
                    "====================================================================================================\n\n");
    }

    void report_best() const
    {
        for (const auto &a : algorithms) {
            std::printf("Optimal setup for algorithm %s:\n\tData layout: %s\n\tWork-group size: %u\n\tAverage total time: %g\n",
                        a.c_str(), best_layout.at(a).c_str(), best_wg.at(a), best_time.at(a));
        }
        if (linear)
            std::printf("Optimal setup for algorithm lptl (Linear Pull Two-Lattice):\n\tData layout: %s\n\tAverage total time: %g\n\n",
                        best_layout.at("lptl").c_str(), best_time.at("lptl"));
    }

    std::vector<std::string> algorithms, layouts, scenarios;
    std::vector<unsigned> wgs;
    bool linear = false;
    std::map<std::string, std::string> best_layout;
    std::map<std::string, unsigned> best_wg;
    std::map<std::string, double> best_time;
    plbm_properties p_{};
    std::string scn_ = "Hagen-Poiseuille";

  private:
    std::string out_, device_, alg_, lay_;
    double hbm_, bytes_node_ = 8;
    unsigned runs_;
    plbm_options opts_{};
};

std::vector<std::string> strings(const Json &j)
{
    std::vector<std::string> out;
    if (j.type != Json::ARRAY) throw plbm::JsonError("type_error: expected an array of strings");
    for (const auto &v : j.arr) out.push_back(v.as_string());
    return out;
}

}  // namespace

extern "C" {

int plbm_benchmark_work_group_sizes(unsigned max_work_group_size, unsigned *out, unsigned capacity, unsigned *count)
{
    const std::vector<unsigned> w = work_group_sizes(max_work_group_size);
    if (count) *count = (unsigned)w.size();
    if (out)
        for (size_t i = 0; i < w.size() && i < capacity; ++i) out[i] = w[i];
    return PLBM_OK;
}

int plbm_benchmark_run(const char *settings_path, const char *benchmark_path, const char *output_root,
                       const plbm_options *opts, unsigned phases, double hbm_gbs)
{
    if (!settings_path) return PLBM_ERR_ARGUMENT;
    // the handler's error string carries the message; plbm_last_error(NULL) reports it
    plbm_properties base{};
    int rc = plbm_json_to_properties(settings_path, -2, &base);   // Benchmark ctor: json_to_properties(path, -2)
    if (rc != PLBM_OK) return rc;
    const fs::path root = fs::absolute(fs::path(settings_path)).parent_path().parent_path();
    const std::string bpath = benchmark_path ? benchmark_path : (root / "settings" / "benchmark.json").string();
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PLBM_ERR_NO_DEVICE;
    const int dev = opts ? opts->device : 0;
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return PLBM_ERR_CUDA;
    try {
        std::ifstream f(bpath);
        if (!f) return PLBM_ERR_IO;
        std::stringstream ss;
        ss << f.rdbuf();
        const std::string text = ss.str();
        const Json b = plbm::JsonParser(text).parse();
        // Benchmark ctor (benchmark.cpp:64-108): no debug output, results only after the last step,
        // the channel scenario for phases 0 and 1
        base.debug_mode = 0;
        base.frame_update_interval = base.time_steps + 1;
        const unsigned runs = b.at("testRunsPerConfig").as_unsigned();
        Bench bench(base, opts, output_root ? output_root : root.string(), prop.name, hbm_gbs, runs);
        bench.algorithms = strings(b.at("algorithms"));
        bench.layouts = strings(b.at("dataLayouts"));
        bench.scenarios = strings(b.at("phaseTwoScenarios"));
        bench.linear = b.at("testLinearTwoLattice").as_bool();
        bench.wgs = work_group_sizes((unsigned)prop.maxThreadsPerBlock);
        for (const auto &a : bench.algorithms) {
            bench.best_layout[a] = "stream";
            bench.best_wg[a] = 1;
            bench.best_time[a] = std::numeric_limits<double>::max();
        }
        bench.best_layout["lptl"] = "stream";
        bench.best_wg["lptl"] = 1;
        bench.best_time["lptl"] = std::numeric_limits<double>::max();
        if (phases == 0) phases = 7;
        std::printf("Starting benchmark.\n\n");
        if (phases & 1) {   // phase_0 (benchmark.cpp:242-248): 10 steps
            const unsigned T = bench.p_.time_steps;
            bench.p_.time_steps = 10;
            bench.p_.frame_update_interval = 11;
            bench.phase_0_1(0);
            bench.p_.time_steps = T;
            bench.p_.frame_update_interval = T + 1;
        }
        if (phases & 2) {
            bench.phase_0_1(1);
            bench.report_best();
        }
        if (phases & 4) bench.phase_2();
        std::printf("\nDone with all benchmarks.\n\n");
        std::fflush(stdout);
    } catch (const plbm::JsonError &e) {
        std::fprintf(stderr, "benchmark settings: %s\n", e.what());
        return PLBM_ERR_PARSE;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "benchmark: %s\n", e.what());
        return PLBM_ERR_IO;
    }
    return PLBM_OK;
}

}  // extern "C"
