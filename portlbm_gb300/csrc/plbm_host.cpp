// plbm_host.cpp — host side of libplbm: the C ABI declared in include/plbm_c.h.
//
// Mirrors, in C++ on top of hand-written sm_103a kernels, the reference's host path
// (SC-SGS/PortLBM): Properties and its validation (src/lbm/core/simulation.cpp:21-125),
// Domain arithmetic (:194-382), settings.json I/O (src/lbm/file_interaction/
// file_interaction.cpp:11-69), geometry set-up (include/lbm/core/domain_initialization.hpp),
// and the SYCLAlgorithmHandler life cycle (include/lbm/execution/sycl_algorithm_handler.hpp:
// 252-455) with its per-step loop (include/lbm/gpu/nptl/nptl.hpp:116-141 and twins).
//
// Differences by design: one fused kernel launch per timestep instead of 3-7 launches each
// followed by a host wait; observables are written on the steps that are copied to the host
// (every other step's values are overwritten before any copy in the reference); runs of steps
// between copies are replayed from a captured CUDA graph.
#include "../../include/plbm_c.h"
#include "plbm_consts.h"
#include "plbm_json.hpp"
#include "plbm_launch.h"
#include "plbm_power.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <future>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

using plbm::Json;
using plbm::JsonError;

struct Status {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string &msg) { throw Status{ code, msg }; }

void cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) fail(PLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// PLBM_TRACE=1 in the environment: handler set-up and runs print the wall-clock milliseconds of
// their phases to stderr (observability; off by default).
struct PhaseTrace {
    bool on;
    const char *what;
    std::chrono::steady_clock::time_point t0;
    explicit PhaseTrace(const char *w) : on(std::getenv("PLBM_TRACE") != nullptr), what(w), t0(std::chrono::steady_clock::now()) {}
    void operator()(const char *phase) const
    {
        if (!on) return;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::fprintf(stderr, "[plbm] %s %s %.2f ms\n", what, phase, ms);
    }
};

// ---- core::Properties (include/lbm/core/properties.hpp:30-166) ---------------------------

struct Props {
    std::string algorithm, data_layout, scenario, settings_path;
    bool debug_mode = false;
    unsigned work_group_size = 0, time_steps = 0, frame_update_interval = 0;
    unsigned vertical_nodes = 0, horizontal_nodes = 0;   // stored extents: inner + 2
    unsigned total_unexpanded_node_count = 0, domain_node_count = 0;
    double ivx = 0, ivy = 0, irho = 0, ovx = 0, ovy = 0, orho = 0, tau = 0;

    // Properties::Properties (simulation.cpp:21-58): inner extents in, ghost layers added.
    static Props make(const plbm_properties &c)
    {
        Props p;
        p.algorithm = c.algorithm ? c.algorithm : "";
        p.data_layout = c.data_layout ? c.data_layout : "";
        p.scenario = c.scenario ? c.scenario : "";
        p.debug_mode = c.debug_mode != 0;
        p.work_group_size = c.work_group_size;
        p.time_steps = c.time_steps;
        p.frame_update_interval = c.frame_update_interval;
        p.vertical_nodes = c.vertical_nodes + 2;
        p.horizontal_nodes = c.horizontal_nodes + 2;
        p.total_unexpanded_node_count = (c.vertical_nodes + 2) * (c.horizontal_nodes + 2);
        p.domain_node_count = c.vertical_nodes * c.horizontal_nodes;
        p.ivx = c.inlet_velocity_x; p.ivy = c.inlet_velocity_y; p.irho = c.inlet_density;
        p.ovx = c.outlet_velocity_x; p.ovy = c.outlet_velocity_y; p.orho = c.outlet_density;
        p.tau = c.relaxation_time;
        return p;
    }

    // Properties::validate (simulation.cpp:60-125), same checks, order and messages.
    void validate() const
    {
        static const char *algs[] = { "nptl", "lptl", "npol", "nsol" };
        static const char *lays[] = { "stream", "collision", "bundle" };
        static const char *scns[] = { "Hagen-Poiseuille", "walls", "circle", "square", "plate", "skyscraper", "wing", "porous" };
        if (vertical_nodes < 4) fail(PLBM_ERR_PROPERTY, "vertical_nodes must be >= 4 (inner domain >= 2 rows)");
        if (horizontal_nodes < 4) fail(PLBM_ERR_PROPERTY, "horizontal_nodes must be >= 4 (inner domain >= 2 cols)");
        if (time_steps < 1) fail(PLBM_ERR_PROPERTY, "time_steps must be >= 1");
        if (frame_update_interval < 1) fail(PLBM_ERR_PROPERTY, "frame_update_interval must be >= 1");
        if (work_group_size < 1) fail(PLBM_ERR_PROPERTY, "work_group_size must be >= 1");
        if (irho <= 0) fail(PLBM_ERR_PROPERTY, "inlet_density must be > 0");
        if (orho <= 0) fail(PLBM_ERR_PROPERTY, "outlet_density must be > 0");
        if (tau <= 0) fail(PLBM_ERR_PROPERTY, "relaxation_time must be > 0");
        auto in = [](const std::string &v, const char *const *l, int n) {
            for (int i = 0; i < n; ++i)
                if (v == l[i]) return true;
            return false;
        };
        if (!in(algorithm, algs, 4))
            fail(PLBM_ERR_PROPERTY, "Unknown algorithm: \"" + algorithm + "\". Valid values: lptl, nptl, npol, nsol");
        if (!in(data_layout, lays, 3))
            fail(PLBM_ERR_PROPERTY,
                 "Unknown data_layout: \"" + data_layout + "\". Valid values: stream, collision, bundle");
        if (!in(scenario, scns, 8))
            fail(PLBM_ERR_PROPERTY, "Unknown scenario: \"" + scenario +
                                        "\". Valid values: Hagen-Poiseuille, walls, circle, square, plate, skyscraper, wing, porous");
    }

    plbm_properties to_c() const
    {
        plbm_properties c{};
        c.algorithm = algorithm.c_str(); c.data_layout = data_layout.c_str(); c.scenario = scenario.c_str();
        c.debug_mode = debug_mode; c.work_group_size = work_group_size; c.time_steps = time_steps;
        c.frame_update_interval = frame_update_interval;
        c.vertical_nodes = vertical_nodes - 2; c.horizontal_nodes = horizontal_nodes - 2;
        c.inlet_velocity_x = ivx; c.inlet_velocity_y = ivy; c.inlet_density = irho;
        c.outlet_velocity_x = ovx; c.outlet_velocity_y = ovy; c.outlet_density = orho;
        c.relaxation_time = tau;
        return c;
    }
};

// ---- settings.json (file_interaction.cpp:11-69) -----------------------------------------

std::string read_file(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) fail(PLBM_ERR_PARSE, "parse_error: cannot open settings file '" + path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// A rows x cols float64 array as a NumPy .npy file (format 1.0, little-endian, C order): the
// headless stand-in for the reference's GUI frames.
bool write_npy(const std::string &path, const double *data, unsigned rows, unsigned cols)
{
    std::string hdr = "{'descr': '<f8', 'fortran_order': False, 'shape': (" + std::to_string(rows) + ", " +
                      std::to_string(cols) + "), }";
    const size_t pre = 10;   // magic (6) + version (2) + header length (2)
    size_t total = pre + hdr.size() + 1;
    hdr.append((64 - total % 64) % 64, ' ');
    hdr += '\n';
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    const unsigned char magic[8] = { 0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0 };
    f.write(reinterpret_cast<const char *>(magic), 8);
    const unsigned short hl = (unsigned short)hdr.size();
    const unsigned char hlb[2] = { (unsigned char)(hl & 0xff), (unsigned char)(hl >> 8) };
    f.write(reinterpret_cast<const char *>(hlb), 2);
    f.write(hdr.data(), (std::streamsize)hdr.size());
    for (size_t i = 0; i < (size_t)rows * cols; ++i) {   // explicit little-endian bytes
        uint64_t u;
        std::memcpy(&u, &data[i], 8);
        unsigned char b[8];
        for (int k = 0; k < 8; ++k) b[k] = (unsigned char)(u >> (8 * k));
        f.write(reinterpret_cast<const char *>(b), 8);
    }
    return (bool)f;
}

struct JsonExtras {
    int precision = -1;
    int nan_protection = -1;
};

int precision_from_name(const std::string &s)
{
    static const char *names[] = { "f64_strict", "f64_fast", "f32_ref", "f32", "f16s", "bf16s", "f64_q60", "f16c" };
    for (int i = 0; i < 8; ++i)
        if (s == names[i]) return i;
    fail(PLBM_ERR_PROPERTY, "Unknown gb300.precision: \"" + s +
                                "\". Valid values: f64_strict, f64_fast, f32_ref, f32, f16s, bf16s, f64_q60, f16c");
}

// json_to_properties(path, offset): the node counts read are inner extents plus `offset`, and the
// Properties constructor adds the two ghost layers.
Props json_to_props(const std::string &path, int offset, JsonExtras *extras)
{
    const std::string text = read_file(path);
    try {
        const Json root = plbm::JsonParser(text).parse();
        const Json &a = root.at("algorithmic"), &d = root.at("domain"), &ph = root.at("physical");
        plbm_properties c{};
        std::string alg = a.at("algorithm").as_string(), lay = a.at("dataLayout").as_string();
        c.debug_mode = a.at("debugMode").as_bool();
        c.work_group_size = a.at("workGroupSize").as_unsigned();
        c.time_steps = a.at("timeSteps").as_unsigned();
        c.frame_update_interval = a.at("frameUpdateInterval").as_unsigned();
        std::string scn = d.at("scenario").as_string();
        c.vertical_nodes = d.at("verticalNodes").as_unsigned() + (unsigned)offset;
        c.horizontal_nodes = d.at("horizontalNodes").as_unsigned() + (unsigned)offset;
        c.inlet_velocity_x = ph.at("inletVelocity").at("x").as_double();
        c.inlet_velocity_y = ph.at("inletVelocity").at("y").as_double();
        c.inlet_density = ph.at("inletDensity").as_double();
        c.outlet_velocity_x = ph.at("outletVelocity").at("x").as_double();
        c.outlet_velocity_y = ph.at("outletVelocity").at("y").as_double();
        c.outlet_density = ph.at("outletDensity").as_double();
        c.relaxation_time = ph.at("relaxationTime").as_double();
        c.algorithm = alg.c_str(); c.data_layout = lay.c_str(); c.scenario = scn.c_str();
        Props p = Props::make(c);
        p.settings_path = path;
        if (extras) {
            if (const Json *g = root.find("gb300")) {
                if (const Json *pr = g->find("precision")) extras->precision = precision_from_name(pr->as_string());
                if (const Json *np = g->find("nanProtection")) extras->nan_protection = np->as_bool() ? 1 : 0;
            }
        }
        return p;
    } catch (const JsonError &e) {
        fail(PLBM_ERR_PARSE, e.what());
    }
}

// properties_to_json (file_interaction.cpp:11-37): writes the given node counts as they are.
void props_to_json(const Props &p, unsigned vnodes, unsigned hnodes, const std::string &path)
{
    Json root;
    Json &a = root.set("algorithmic");
    a.set("workGroupSize") = plbm::jnum(p.work_group_size, true);
    a.set("debugMode") = plbm::jbool(p.debug_mode);
    a.set("timeSteps") = plbm::jnum(p.time_steps, true);
    a.set("dataLayout") = plbm::jstr(p.data_layout);
    a.set("algorithm") = plbm::jstr(p.algorithm);
    a.set("frameUpdateInterval") = plbm::jnum(p.frame_update_interval, true);
    Json &d = root.set("domain");
    d.set("scenario") = plbm::jstr(p.scenario);
    d.set("verticalNodes") = plbm::jnum(vnodes, true);
    d.set("horizontalNodes") = plbm::jnum(hnodes, true);
    Json &ph = root.set("physical");
    Json &iv = ph.set("inletVelocity");
    iv.set("x") = plbm::jnum(p.ivx, false);
    iv.set("y") = plbm::jnum(p.ivy, false);
    ph.set("inletDensity") = plbm::jnum(p.irho, false);
    Json &ov = ph.set("outletVelocity");
    ov.set("x") = plbm::jnum(p.ovx, false);
    ov.set("y") = plbm::jnum(p.ovy, false);
    ph.set("outletDensity") = plbm::jnum(p.orho, false);
    ph.set("relaxationTime") = plbm::jnum(p.tau, false);
    std::string out;
    plbm::json_dump(out, root);
    std::ofstream f(path);
    f << out;
}

// ---- core::Domain (simulation.cpp:194-382; power functions simulation.hpp:373-446) -----------

struct Domain {
    unsigned total_node_count, horizontal_nodes, vertical_nodes, subdomain_vertical_nodes,
        subdomain_horizontal_nodes, subdomain_count_vertical, subdomain_count_horizontal;
};

using plbm::which_power_of_4;
using plbm::which_power_of_2;

void power_of_two_handling(size_t wg, unsigned &sv, unsigned &sh)
{
    const size_t p4 = which_power_of_4(wg), p2 = which_power_of_2(wg);
    if (p4) {
        size_t size = 1;
        for (size_t i = 0; i < p4; ++i) size *= 2;
        sh = sv = (unsigned)size;
    } else if (p2) {
        size_t height = 1;
        for (size_t i = 0; i < p2 / 2; ++i) height *= 2;
        sv = (unsigned)height;
        sh = (unsigned)(2 * height);
    } else {
        sv = 2;
        sh = (unsigned)(wg / 2);
    }
}

void subdomain_count(unsigned ext, unsigned sub, unsigned &c)
{
    c = ((ext - 2) / sub) + 1;
    if (!((ext - 2) % sub)) c--;
}

// Returns false when nsol's work-group size is below its minimum of 6.
bool make_domain(const Props &p, Domain &d)
{
    const unsigned X = p.horizontal_nodes, V = p.vertical_nodes;
    d = Domain{ X * V, X, V, V, X, 1, 1 };
    if (p.algorithm == "lptl") return true;
    unsigned sv, sh;
    size_t w = p.work_group_size;
    if (p.algorithm == "nsol") {
        if (w < 6) return false;
        if (w & 0x1) w--;
        power_of_two_handling(w, sv, sh);
        sv -= 1;
        sh -= 2;
        // setup_for_swap with 2x2 tiles (which_power_of_4 returns 1, e.g. wg 20 or 100) leaves an
        // empty subdomain and the reference divides by zero; refuse the size instead.
        if (sh == 0 || sv == 0)
            fail(PLBM_ERR_PROPERTY, "work-group size " + std::to_string(p.work_group_size) +
                                        " gives the swap algorithm an empty subdomain (2x2 tiles minus its halo)");
    } else if (w & 0x1) {
        sh = (unsigned)w;
        sv = 1;
    } else {
        power_of_two_handling(w, sv, sh);
    }
    d.subdomain_vertical_nodes = sv;
    d.subdomain_horizontal_nodes = sh;
    subdomain_count(V, sv, d.subdomain_count_vertical);
    subdomain_count(X, sh, d.subdomain_count_horizontal);
    if (p.algorithm == "nptl") {
        d.vertical_nodes = sv * d.subdomain_count_vertical + 2;
        d.horizontal_nodes = sh * d.subdomain_count_horizontal + 2;
    } else {
        d.vertical_nodes = (sv + 1) * d.subdomain_count_vertical + 1;
        d.horizontal_nodes = (sh + 1) * d.subdomain_count_horizontal + 1;
    }
    d.total_node_count = d.vertical_nodes * d.horizontal_nodes;
    return true;
}

// ---- geometry (domain_initialization.hpp:41-297, :453-518) -------------------------------

unsigned stencil(const std::string &sc, unsigned x, unsigned y, unsigned V, unsigned X)
{
    if (sc == "walls") {
        unsigned cond = (x == (1 * X) / 6 || x == (3 * X) / 6 || x == (5 * X) / 6) && (y > 1) && (y < V / 2);
        cond += (x == (2 * X) / 6 || x == (4 * X) / 6) && (y < V - 2) && (y > ((V - 1) / 2));
        return cond;
    }
    if (sc == "circle") {
        const unsigned mx = 2 * X / 10, my = V / 2, r = V / 5, dx = mx - x, dy = my - y;
        return (y >= my - r) && (y <= my + r) && (x >= mx - r) && (x <= mx + r) && (dx * dx + dy * dy <= r * r);
    }
    if (sc == "square") {
        const unsigned mx = 2 * X / 10, my = V / 2, hl = V / 10;
        return (y >= my - hl) && (y <= my + hl) && (x >= mx - hl) && (x <= mx + hl);
    }
    if (sc == "plate") {
        const unsigned mx = X / 10, my = V / 2, hh = 7 * V / 40, hw = hh / 60;
        return (y >= my - hh) && (y <= my + hh) && (x >= mx - hw) && (x <= mx + hw);
    }
    if (sc == "skyscraper") {
        const unsigned ha = V / 2, hwa = 1, hs = 2 * V / 5, hws = V / 24, hf = V / 4, hwf = V / 16, mx = 3 * X / 10;
        return ((y >= 1) && (y <= hf && x >= mx - hwf && x <= mx + hwf)) ||
               (y <= hs && x >= mx - hws && x <= mx + hws) || (y <= ha && x >= mx - hwa && x <= mx + hwa);
    }
    if (sc == "wing") {
        const int mx = (int)(X / 5), my = (int)(V / 2), rmax = (int)(V / 5), sy = 5;
        const unsigned ddx = x - (unsigned)mx, ddy = y - (unsigned)my;
        return ((0.2 * (double)(ddx * ddx) + (double)(ddy * ddy)) <= rmax) ||
               ((std::pow((double)ddx, 1.4) + (double)((unsigned)(sy * sy) * (ddy * ddy))) <= sy * sy * rmax);
    }
    return 0;  // Hagen-Poiseuille
}

// Inner W*H flag grid (0 fluid, 1 solid) in reference coordinates (x, y) -> (x-1, y-1).
std::vector<int8_t> make_flags(const Props &p, const std::vector<int8_t> *mask)
{
    const unsigned X = p.horizontal_nodes, V = p.vertical_nodes, W = X - 2, H = V - 2;
    std::vector<int8_t> f((size_t)W * H, -1);
    auto at = [&](unsigned x, unsigned y) -> int8_t & { return f[(size_t)(x - 1) + (size_t)(y - 1) * W]; };
    if (mask) {
        for (size_t i = 0; i < f.size(); ++i) f[i] = (*mask)[i];
        return f;
    }
    if (p.scenario == "porous") {
        // porous_medium_mask :265-297 draws from the process-wide std::rand() sequence.
        for (int y = 2; (unsigned)y < V - 2; ++y)
            for (int x = 1; (unsigned)x <= X - 2; ++x) {
                const int one = 1 + (std::rand() % 10), two = 1 + (std::rand() % 10);
                at((unsigned)x, (unsigned)y) = (x % one == one - 1 && y % two == two - 1) ? 1 : 0;
            }
        for (int y = 1; (unsigned)y < V; y += (int)(V - 3))
            for (int x = 1; (unsigned)x <= X - 2; ++x)
                if ((unsigned)y <= V - 2) at((unsigned)x, (unsigned)y) = 1;
        return f;
    }
    for (unsigned x = 1; x <= X - 2; ++x) { at(x, 1) = 1; at(x, V - 2) = 1; }   // set_pipe_boundaries :214-239
    for (unsigned y = 2; y + 2 < V; ++y)                                         // add_stencil :414-440
        for (unsigned x = 1; x + 1 < X; ++x) at(x, y) = (int8_t)stencil(p.scenario, x, y, V, X);
    return f;
}

int alg_index(const std::string &a) { return a == "nptl" ? 0 : a == "lptl" ? 1 : a == "npol" ? 2 : 3; }
int layout_index(const std::string &l) { return l == "collision" ? 0 : l == "stream" ? 1 : 2; }
size_t storage_bytes(int prec) { return (prec <= 1 || prec == PLBM_F64_Q60) ? 8 : prec <= 3 ? 4 : 2; }

using plbm::maxwell_boltzmann;

thread_local std::string g_tls_error;
std::mutex g_create_mu;
std::string g_create_error;

}  // namespace

// Host result arrays: allocation alignment (the largest base page size of the supported hosts).
static constexpr size_t HOST_ALIGN = 65536;

// Sets the four result arrays to their initial values (rho = -1, j = 0), the pages first touched
// by up to 16 threads: writing gigabytes of fresh pages is bound by the kernel's page zeroing,
// which scales with the threads.
static void parallel_fill(double *const res[4], size_t n)
{
    const size_t bytes = 4 * n * sizeof(double);
    unsigned nt = bytes < (64u << 20) ? 1u : std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    auto fill = [&](unsigned t) {
        for (int i = 0; i < 4; ++i) {
            const size_t a = n * t / nt, b = n * (t + 1) / nt;
            std::fill(res[i] + a, res[i] + b, i == 0 ? -1.0 : 0.0);
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(fill, t);
    fill(0);
    for (auto &th : pool) th.join();
}

// ---- the handler --------------------------------------------------------------------------

struct plbm_handler {
    Props props;
    std::string settings_path;
    bool from_json = false;
    plbm_options opt{};
    bool opt_precision_set = false;
    // A caller's mask is uploaded once, from the caller's buffer during plbm_create, into mask_d,
    // which stays on the device for later initialize() calls (a host copy of an 8192^2 mask would
    // cost more than the whole device set-up).
    const int8_t *mask_src = nullptr;   // the caller's mask during plbm_create
    int8_t *mask_d = nullptr;
    size_t mask_n = 0;
    bool has_mask = false;
    Domain dom{};
    int alg = 0, lay = 0, prec = 0;
    int W = 0, H = 0, P = 0;
    unsigned long long N = 0;
    int outlet_mode = 0;
    // debugMode on nptl / lptl: the reference's unfused stream / observables / collide kernels
    bool debug = false;
    bool porous = false;   // nptl/lptl shifted forms: the obstacle-select gather (PLBM_GATHER_POROUS)

    cudaStream_t stream = nullptr;
    void *lat[2] = { nullptr, nullptr };
    uint16_t *links = nullptr;
    int8_t *flags_d = nullptr;
    double *res_d[4] = { nullptr, nullptr, nullptr, nullptr };
    double *jy_d = nullptr;
    void *halo[2] = { nullptr, nullptr };
    double *red_d = nullptr;
    int *status_d = nullptr;
    double *jprev_d = nullptr;   // 2 * W*H: j of the previous residual evaluation
    long long jprev_iter = -1;   // iteration at which jprev_d was taken (-1: none)
    std::string export_dir;      // frame export (empty: off)
    unsigned export_fields = 0;  // bit i: result i (PLBM_DENSITY ..)
    double *res_h[4] = { nullptr, nullptr, nullptr, nullptr };
    double *res_hd[4] = { nullptr, nullptr, nullptr, nullptr };   // device addresses of res_h
    // a result step wrote res_h through res_hd (the step loop's frames): res_d is older than res_h
    std::atomic<bool> host_results_newer{ false };
    size_t res_h_bytes = 0;
    bool res_h_registered = false;
    // The host result arrays are allocated, first touched with their initial values by parallel
    // threads and then registered with the driver (page-locked, device-mapped), all on a host
    // thread while the device is set up and stepping; every access waits for it (wait_host()).
    // cudaMallocHost would zero and lock the same pages on one thread while holding the driver's
    // lock, stalling the device set-up behind it (~70 ms for the four 537 MB arrays of 8192^2).
    std::future<std::string> host_ready;
    std::mutex host_mu;            // the step-loop thread and a caller's getter may both wait
    std::string host_err;

    std::string join_host()
    {
        std::lock_guard<std::mutex> g(host_mu);
        if (host_ready.valid()) host_err = host_ready.get();
        return host_err;
    }
    void wait_host()
    {
        const std::string err = join_host();
        if (!err.empty()) fail(PLBM_ERR_CUDA, err);
    }
    size_t nres = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    plbm::StepParams base{};
    dim3 grid, block;
    cudaGraphExec_t gexec = nullptr;
    cudaGraphExec_t frame_gexec[2] = { nullptr, nullptr };   // one frame, by starting parity
    unsigned frame_graph_len = 0;
    unsigned graph_steps = 0;

    std::atomic<unsigned> iteration{ 0 };
    std::atomic<bool> stop{ false };
    std::atomic<double> progress{ 0.0 };
    std::atomic<double> frametime{ 1.7976931348623157e308 };
    std::thread worker;
    bool active = false;
    bool future_valid = true;
    std::mutex mu;
    int worker_status = PLBM_OK;
    std::string worker_error;
    std::string last_error;

    ~plbm_handler()
    {
        release();
        if (mask_d) cudaFree(mask_d);
    }

    void release()
    {
        if (worker.joinable()) { stop = true; worker.join(); }
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        for (auto &f : frame_gexec) { if (f) cudaGraphExecDestroy(f); f = nullptr; }
        frame_graph_len = 0;
        for (auto &p : lat) { if (p) cudaFree(p); p = nullptr; }
        for (auto &p : halo) { if (p) cudaFree(p); p = nullptr; }
        for (auto &p : res_d) { if (p) cudaFree(p); p = nullptr; }
        join_host();
        host_err.clear();
        for (int i = 0; i < 4; ++i) {
            if (res_h[i] && res_h_registered) cudaHostUnregister(res_h[i]);
            std::free(res_h[i]);
            res_h[i] = nullptr;
            res_hd[i] = nullptr;
        }
        res_h_registered = false;
        if (links) cudaFree(links);
        if (flags_d) cudaFree(flags_d);
        if (jy_d) cudaFree(jy_d);
        if (red_d) cudaFree(red_d);
        if (status_d) cudaFree(status_d);
        if (jprev_d) cudaFree(jprev_d);
        jprev_d = nullptr;
        links = nullptr; flags_d = nullptr; jy_d = nullptr; red_d = nullptr; status_d = nullptr;
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        ev0 = ev1 = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    bool two_lattice() const { return alg == 0 || alg == 1; }

    // SYCLAlgorithmHandler::initialize_algorithm (:252-272) + core::Simulation (simulation.cpp:
    // 438-519) + setup_domain (domain_initialization.hpp:453-518).
    void build()
    {
        const PhaseTrace trace("create");
        release();
        iteration = 0; progress = 0.0; frametime = 1.7976931348623157e308; jprev_iter = -1;
        stop = false; active = false; future_valid = true; worker_status = PLBM_OK; worker_error.clear();
        JsonExtras ex;
        if (from_json) props = json_to_props(settings_path, 0, &ex);
        // SYCLAlgorithmHandler::initialize_non_debug_algorithm (:75-157) rejects unknown names
        // with exceptions::Exception; the remaining checks are Properties::validate()'s.
        if (props.algorithm != "nptl" && props.algorithm != "lptl" && props.algorithm != "npol" && props.algorithm != "nsol")
            fail(PLBM_ERR_UNKNOWN, "Unknown algorithm: " + props.algorithm);
        if (props.data_layout != "stream" && props.data_layout != "collision" && props.data_layout != "bundle")
            fail(PLBM_ERR_UNKNOWN, "Unknown data layout: " + props.data_layout);
        props.validate();
        prec = opt.precision;
        if (ex.precision >= 0 && !opt_precision_set) prec = ex.precision;
        if (ex.nan_protection >= 0) opt.nan_protection = ex.nan_protection;
        if (prec < 0 || prec > 7) fail(PLBM_ERR_ARGUMENT, "precision must be one of PLBM_F64_STRICT..PLBM_F16C");
        // NPTLDebug / LPTLDebug run unfused kernels (sycl_algorithm_handler.hpp:164-246); NPOLDebug
        // and NSOLDebug keep the fused step, as here
        debug = props.debug_mode && (props.algorithm == "nptl" || props.algorithm == "lptl");
        if (debug && prec != PLBM_F64_STRICT && prec != PLBM_F32_REF)
            fail(PLBM_ERR_ARGUMENT, "debugMode runs the reference's unfused kernels, in the f64_strict or f32_ref "
                                    "form only");

        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) fail(PLBM_ERR_NO_DEVICE, "no CUDA device available");
        cuda_check(cudaSetDevice(opt.device), "cudaSetDevice");
        int max_wg = 0;
        cuda_check(cudaDeviceGetAttribute(&max_wg, cudaDevAttrMaxThreadsPerBlock, opt.device), "device attribute");
        if (props.work_group_size > (unsigned)max_wg) {
            const unsigned wrong = props.work_group_size;
            if (from_json) {   // simulation.cpp:445-459: rewrite settings.json, then throw
                Props q = props;
                q.work_group_size = (unsigned)max_wg;
                props_to_json(q, q.vertical_nodes - 2, q.horizontal_nodes - 2, settings_path);
                fail(PLBM_ERR_PROPERTY, "Detected illegal work group size of " + std::to_string(wrong) +
                                            " that exceeds the maximum work group size of " + std::to_string(max_wg) +
                                            ". JSON property \"workGroupSize\" has been set to " + std::to_string(max_wg) +
                                            " to enable graceful program restart. ");
            }
            fail(PLBM_ERR_PROPERTY, "work_group_size " + std::to_string(wrong) + " exceeds the device maximum of " +
                                        std::to_string(max_wg) + "; reduce it to " + std::to_string(max_wg) +
                                        " and reconstruct.");
        }
        if (!make_domain(props, dom)) {
            // setup_for_swap simulation.cpp:336-353: re-read the settings, set 6, write back, throw.
            if (props.settings_path.empty())
                fail(PLBM_ERR_PARSE, "parse_error: settings file '' cannot be read to correct workGroupSize");
            Props q = json_to_props(props.settings_path, -2, nullptr);
            q.work_group_size = 6;
            props_to_json(q, q.vertical_nodes, q.horizontal_nodes, props.settings_path);
            fail(PLBM_ERR_PROPERTY, "Detected illegal work group size of " + std::to_string(props.work_group_size) +
                                        " that is below the minimum work-group size of 6 of the swap algorithm. JSON "
                                        "property \"workGroupSize\" has been set to 6 to enable graceful program restart. ");
        }
        alg = alg_index(props.algorithm);
        lay = layout_index(props.data_layout);
        W = (int)props.horizontal_nodes - 2;
        H = (int)props.vertical_nodes - 2;
        P = (W + 31) / 32 * 32;
        N = (unsigned long long)P * H;
        nres = (size_t)W * H;
        // Buffered outlet border lookup (buffered.hpp:285-288): the border is taken as
        // BufferedNodeAccess(X-3, y) + 1, which is a buffer column when (X-3) is a multiple of the
        // subdomain width; the outlet's writes then land on the border nodes' own populations
        // (overwritten by their collision) and the outlet ghost keeps feq(outlet).
        outlet_mode = 0;
        if ((alg == 2 || alg == 3) && ((props.horizontal_nodes - 3) % dom.subdomain_horizontal_nodes) == 0) outlet_mode = 1;

        if (has_mask && mask_n != nres) fail(PLBM_ERR_ARGUMENT, "mask must hold inner W*H entries");
        // a caller's mask is uploaded as it is (its 0/1 values are checked on the device below);
        // otherwise the scenario's flags are built on the host
        std::vector<int8_t> flags;
        if (!has_mask) flags = make_flags(props, nullptr);
        const int8_t *flags_src = has_mask ? mask_d : flags.data();

        trace("host checks");
        cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
        cuda_check(cudaEventCreate(&ev0), "event");
        cuda_check(cudaEventCreate(&ev1), "event");
        const size_t eb = storage_bytes(prec);
        const size_t lat_bytes = 9ull * N * eb;
        size_t free_b = 0, total_b = 0;
        cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
        const size_t need = lat_bytes * (two_lattice() ? 2 : 1) + N * 2 + nres * (1 + 4 * 8);
        if (need + (256ull << 20) > free_b)
            fail(PLBM_ERR_CUDA, "out of device memory: need " + std::to_string(need >> 20) + " MiB, free " +
                                    std::to_string(free_b >> 20) + " MiB");
        for (int i = 0; i < (two_lattice() ? 2 : 1); ++i) cuda_check(cudaMalloc(&lat[i], lat_bytes), "cudaMalloc lattice");
        cuda_check(cudaMalloc(&links, N * sizeof(uint16_t)), "cudaMalloc links");
        cuda_check(cudaMalloc(&flags_d, nres), "cudaMalloc flags");
        for (auto &r : res_d) cuda_check(cudaMalloc(&r, nres * sizeof(double)), "cudaMalloc results");
        trace("device allocations");
        host_ready = std::async(std::launch::async, [this, dev = opt.device, trace]() -> std::string {
            res_h_bytes = (nres * sizeof(double) + HOST_ALIGN - 1) / HOST_ALIGN * HOST_ALIGN;
            for (auto &r : res_h) {
                r = static_cast<double *>(std::aligned_alloc(HOST_ALIGN, res_h_bytes));
                if (!r) return "out of host memory for the results";
            }
            // initial results: rho = -1, j = 0 (simulation.cpp:386-417)
            parallel_fill(res_h, nres);
            trace("host results filled");
            if (cudaSetDevice(dev) != cudaSuccess) return "cudaSetDevice (host results)";
            for (int i = 0; i < 4; ++i) {
                if (cudaHostRegister(res_h[i], res_h_bytes, cudaHostRegisterMapped) != cudaSuccess)
                    return "cudaHostRegister results";
                res_h_registered = true;
                if (cudaHostGetDevicePointer((void **)&res_hd[i], res_h[i], 0) != cudaSuccess)
                    return "cudaHostGetDevicePointer results";
            }
            trace("host results ready");
            return std::string();
        });
        cuda_check(cudaMalloc(&jy_d, 2ull * H * sizeof(double)), "cudaMalloc jy");
        cuda_check(cudaMemsetAsync(jy_d, 0, 2ull * H * sizeof(double), stream), "memset jy");
        cuda_check(cudaMalloc(&red_d, 3 * sizeof(double)), "cudaMalloc reduce");
        cuda_check(cudaMalloc(&status_d, sizeof(int)), "cudaMalloc status");
        cuda_check(cudaMemsetAsync(status_d, 0, sizeof(int), stream), "memset status");
        if (has_mask && !mask_d) {
            cuda_check(cudaMalloc(&mask_d, mask_n), "cudaMalloc mask");
            cuda_check(cudaMemcpyAsync(mask_d, mask_src, mask_n, cudaMemcpyHostToDevice, stream), "H2D mask");
            flags_src = mask_d;
        }
        cuda_check(cudaMemcpyAsync(flags_d, flags_src, nres, has_mask ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                   stream), "flags");
        if (has_mask) cuda_check(plbm::launch_check_mask(flags_d, nres, status_d, stream), "mask check");
        cuda_check(plbm::launch_links(flags_d, links, W, H, P, stream), "links kernel");
        // only the shifted forms of nptl/lptl have a porous instantiation
        const bool has_porous =
            alg <= 1 && (prec == PLBM_F32 || prec == PLBM_F16S || prec == PLBM_BF16S || prec == PLBM_F16C);
        const bool count_obstacles = has_porous && opt.gather == PLBM_GATHER_AUTO;
        if (count_obstacles)   // read after the initialisation sync below
            cuda_check(plbm::launch_count_obstacle_nodes(links, W, H, P, reinterpret_cast<unsigned long long *>(red_d),
                                                         stream), "obstacle count");
        cuda_check(plbm::launch_fill_results(res_d[0], res_d[1], res_d[2], res_d[3], nres, stream), "results fill");
        trace("mask upload and geometry kernels queued");

        // Ghost constants and rest state in the arithmetic of the chosen form.
        plbm::StepParams &b = base;
        std::memset(&b, 0, sizeof b);
        if (prec != PLBM_F32_REF) {
            // double constants; the FP32/FP16/BF16 forms round (feq - w) once, from double
            maxwell_boltzmann<double>(0, 0, 1, b.weight);
            maxwell_boltzmann<double>(props.ivx, props.ivy, props.irho, b.feq_in);
            maxwell_boltzmann<double>(props.ovx, props.ovy, props.orho, b.feq_out);
            b.omega = 1 / props.tau;
            b.rho_out = props.orho;
        } else {
            // the reference's USE_FLOAT build: real_type float throughout
            float w[9], fi[9], fo[9];
            maxwell_boltzmann<float>(0, 0, 1, w);
            maxwell_boltzmann<float>((float)props.ivx, (float)props.ivy, (float)props.irho, fi);
            maxwell_boltzmann<float>((float)props.ovx, (float)props.ovy, (float)props.orho, fo);
            for (int d = 0; d < 9; ++d) { b.weight[d] = w[d]; b.feq_in[d] = fi[d]; b.feq_out[d] = fo[d]; }
            b.omega = (double)(1 / (float)props.tau);
            b.rho_out = (double)(float)props.orho;
        }
        const bool shifted = prec == PLBM_F32 || prec == PLBM_F16S || prec == PLBM_BF16S || prec == PLBM_F16C;
        // the shifted forms keep deviations from w_d * rho0(x'): the straight inlet-outlet profile
        // for the two-lattice pull schemes, rho0 = 1 for npol/nsol
        b.W = W;
        plbm::fill_float_constants(b, shifted, two_lattice(), props.irho, props.orho,
                                   prec == PLBM_F16S ? (double)plbm::F16_SCALE : 1.0);
        {
            plbm::fill_q60_constants(b);
            b.status = status_d;
            if (prec == PLBM_F16C) {
                // the stored deviations of the boundary constants and of the rest state must fit
                // the format (|df| < 0.5); a run that leaves the range later sets the status word
                double worst = 0;
                for (int d = 0; d < 9; ++d) {
                    worst = std::max({ worst, std::fabs((double)b.weightf[d]), std::fabs((double)b.feq_inf[d]),
                                       std::fabs((double)b.feq_outf[d]),
                                       std::fabs((double)b.weightf[d] + (double)b.shift_wg[d] * (W - 1)) });
                }
                if (!(worst < 0.5))
                    fail(PLBM_ERR_NUMERIC, "f16c stores deviations |f - w rho0| < 0.5; these boundary densities "
                                           "exceed it (use f32 or f16s)");
            }
            if (prec == PLBM_F64_Q60) {
                if (!(props.tau > 0.5))
                    fail(PLBM_ERR_NUMERIC, "f64_q60 needs relaxation_time > 0.5 (omega/2 below 1); use f64_strict");
                for (int d = 0; d < 9; ++d)
                    if (std::fabs(b.feq_in[d]) >= 4 || std::fabs(b.feq_out[d]) >= 4)
                        fail(PLBM_ERR_NUMERIC, "f64_q60 needs boundary populations in [-4, 4); use f64_strict");
            }
        }
        double rest[9];
        for (int d = 0; d < 9; ++d) rest[d] = b.weight[d];
        for (int i = 0; i < (two_lattice() ? 2 : 1); ++i) {
            if (shifted)   // rest state rho = 1: w_d (1 - rho0(x'))
                cuda_check(plbm::launch_fill_shifted(lat[i], prec, lay, P, N, rest, b.shift_a, b.shift_g, stream),
                           "lattice fill");
            else
                cuda_check(plbm::launch_fill_lattice(lat[i], prec, lay, N, rest, stream), "lattice fill");
        }

        b.links = links;
        b.rho = res_d[0]; b.jx = res_d[1]; b.jy = res_d[2]; b.jabs = res_d[3];
        b.W = W; b.H = H; b.P = P; b.N = N;
        b.lat_elems = 9ull * N;
        b.outlet_mode = outlet_mode;
        b.nan_protection = opt.nan_protection;

        // Launch shapes.  workGroupSize is honoured as a tile hint (core::Domain's subdomain shape),
        // clamped to what the kernels can run; results do not depend on it.
        const unsigned sh = dom.subdomain_horizontal_nodes, sv = dom.subdomain_vertical_nodes;
        const int cap = plbm::max_threads_for(alg, prec, lay);
        const unsigned ny = (alg == 0 || alg == 1) ? (unsigned)plbm::rows_per_thread(prec) : 1u;
        if (alg == 1) {
            unsigned t = std::min<unsigned>(std::max<unsigned>(props.work_group_size, 32u), (unsigned)cap);
            t = (t + 31) / 32 * 32;
            block = dim3(t);
            grid = dim3((unsigned)((N + (unsigned long long)t * ny - 1) / ((unsigned long long)t * ny)));
        } else {
            // nptl in the stream and bundle layouts: rows of up to 128 nodes per block (measured
            // faster than the subdomain's 32 for the float forms, equal for f64_q60; the collision
            // layout measured 5 % slower with them); the hint sets the height
            unsigned bx = alg == 0 && lay != 0 ? std::min(128u, (unsigned)((W + 31) / 32 * 32))
                                               : alg == 0 || alg == 3 ? std::max(32u, std::min(sh, 128u))
                                                                      : std::min(sh, 64u);
            bx = std::max(1u, bx);
            unsigned by = std::max(1u, std::min(sv, (unsigned)cap / bx));
            if (alg == 2) {   // npol: one tile per block; tile edges carry the halo snapshots
                bx = std::min(bx, (unsigned)W);
                by = std::min(by, (unsigned)H);
            }
            if (alg == 3 && lay == plbm::COLLISION) {   // nsol records: 32 x 8 tiles stage the even step's stores
                bx = 32;
                by = (unsigned)plbm::NSOL_STAGE_ROWS;
            }
            block = dim3(bx, by);
            grid = dim3((W + bx - 1) / bx, (H + by * ny - 1) / (by * ny));
        }
        if (alg == 2) {
            b.tile_w = (int)block.x;
            b.tile_h = (int)block.y;
            b.n_col_bounds = (int)grid.x - 1;
            b.n_row_bounds = (int)grid.y - 1;
            const size_t hn = (size_t)b.n_col_bounds * H * 6 + (size_t)b.n_row_bounds * W * 6;
            b.halo_elems = hn;
            for (auto &hp : halo) {
                cuda_check(cudaMalloc(&hp, std::max<size_t>(hn, 1) * eb), "cudaMalloc halo");
                cuda_check(plbm::launch_fill_halo(hp, prec, W, H, b.n_col_bounds, b.n_row_bounds, rest, stream),
                           "halo fill");
            }
        }
        trace("initialisation queued");
        cuda_check(cudaStreamSynchronize(stream), "initialisation");
        trace("initialisation done");
        porous = has_porous && opt.gather == PLBM_GATHER_POROUS;
        if (count_obstacles) {
            unsigned long long c[2] = { 0, 0 };
            cuda_check(cudaMemcpy(c, red_d, sizeof c, cudaMemcpyDeviceToHost), "obstacle count");
            porous = (double)c[1] > PLBM_GATHER_POROUS_FRACTION * (double)c[0];
        }
        if (has_mask) {
            int bad = 0;
            cuda_check(cudaMemcpy(&bad, status_d, sizeof(int), cudaMemcpyDeviceToHost), "mask check");
            if (bad) fail(PLBM_ERR_ARGUMENT, "mask entries must be 0 (fluid) or 1 (solid)");
        }
        trace("ready");
    }

    // to_host: the step writes its observables straight into the pinned host arrays (device
    // accessible on this platform) instead of the device arrays.
    cudaError_t launch_step(unsigned t, bool results, bool to_host = false)
    {
        plbm::StepParams p = base;
        const unsigned par = t & 1u;
        p.write_results = results ? 1 : 0;
        if (to_host) { p.rho = res_hd[0]; p.jx = res_hd[1]; p.jy = res_hd[2]; p.jabs = res_hd[3]; }
        p.lat0 = two_lattice() ? lat[par] : lat[0];
        p.lat1 = two_lattice() ? lat[par ^ 1u] : nullptr;
        p.jy_prev = jy_d + (size_t)par * H;
        p.jy_next = jy_d + (size_t)(par ^ 1u) * H;
        if (alg == 2) { p.halo_in = (double *)halo[par]; p.halo_out = (double *)halo[par ^ 1u]; }
        if (debug) return plbm::launch_debug_step(prec, lay, alg == 1, p, block, stream);
        switch (alg) {
        case 0: return plbm::launch_nptl(prec, lay, p, grid, block, stream, porous);
        case 1: return plbm::launch_lptl(prec, lay, p, grid, block, stream, porous);
        case 2: return plbm::launch_npol(prec, lay, p, grid, block, stream);
        default: return plbm::launch_nsol(prec, lay, p, t, grid, block, stream);
        }
    }

    // Captures `pairs` (even, odd) step pairs without result writes into one executable graph.
    void ensure_graph()
    {
        if (gexec || !opt.use_graph) return;
        const unsigned pairs = N >= (1ull << 22) ? 4 : 32;
        cudaGraph_t g = nullptr;
        cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        cudaError_t e = cudaSuccess;
        for (unsigned k = 0; k < 2 * pairs && e == cudaSuccess; ++k) e = launch_step(k, false);
        cudaError_t e2 = cudaStreamEndCapture(stream, &g);
        cuda_check(e, "capture launch");
        cuda_check(e2, "end capture");
        cuda_check(cudaGraphInstantiate(&gexec, g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        graph_steps = 2 * pairs;
    }

    // One frame as a graph: F steps, the last writing its results straight into the pinned host
    // arrays; captured once per starting parity and replayed for every full frame but the last
    // (which also refreshes the device result arrays).
    cudaGraphExec_t frame_graph(unsigned t0, unsigned F)
    {
        const unsigned par = t0 & 1u;
        if (frame_graph_len != F) {
            for (auto &f : frame_gexec) { if (f) cudaGraphExecDestroy(f); f = nullptr; }
            frame_graph_len = F;
        }
        if (frame_gexec[par]) return frame_gexec[par];
        wait_host();   // the copies target the pinned host arrays
        cudaGraph_t g = nullptr;
        cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        cudaError_t e = cudaSuccess;
        for (unsigned k = 0; k < F && e == cudaSuccess; ++k) e = launch_step(t0 + k, k + 1 == F, k + 1 == F);
        cudaError_t e2 = cudaStreamEndCapture(stream, &g);
        cuda_check(e, "frame capture");
        cuda_check(e2, "end capture");
        cuda_check(cudaGraphInstantiate(&frame_gexec[par], g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        return frame_gexec[par];
    }

    // Steps [t0, t1) with no result writes; graph replays where the parity allows.
    void run_plain(unsigned t0, unsigned t1)
    {
        unsigned t = t0;
        if (opt.use_graph && t1 - t0 >= 8) {
            ensure_graph();
            if (t & 1u) { cuda_check(launch_step(t, false), "step"); ++t; }
            while (t + graph_steps <= t1) {
                cuda_check(cudaGraphLaunch(gexec, stream), "graph launch");
                t += graph_steps;
            }
        }
        for (; t < t1; ++t) cuda_check(launch_step(t, false), "step");
    }

    // The Q60 form records a population that left its fixed-point range in a device word.
    void check_status()
    {
        if (prec != PLBM_F64_Q60 && prec != PLBM_F16C && !plbm::CHECKED_BUILD) return;
        int st = 0;
        cuda_check(cudaMemcpyAsync(&st, status_d, sizeof(int), cudaMemcpyDeviceToHost, stream), "status");
        cuda_check(cudaStreamSynchronize(stream), "status");
        if (st & plbm::STATUS_OUT_OF_RANGE)
            fail(PLBM_ERR_CUDA, "checked build: a step kernel computed an index outside its buffer (the access was "
                                "skipped)");
        if (st && prec == PLBM_F16C)
            fail(PLBM_ERR_NUMERIC, "a population deviation left the f16c range (-0.5, 0.5) (unstable run?); rerun "
                                   "with f32 or f16s");
        if (st)
            fail(PLBM_ERR_NUMERIC, "a population left the f64_q60 range [-4, 4) (unstable run?); rerun with f64_strict");
    }

    // Frame export: the results of iteration `it` as <dir>/frame_<it>_<field>.npy (H x W).
    void export_frame(unsigned it)
    {
        wait_host();
        static const char *names[4] = { "rho", "jx", "jy", "jabs" };
        char num[16];
        std::snprintf(num, sizeof num, "%09u", it);
        for (int i = 0; i < 4; ++i) {
            if (!(export_fields & (1u << i))) continue;
            const std::string path = export_dir + "/frame_" + num + "_" + names[i] + ".npy";
            if (!write_npy(path, res_h[i], (unsigned)H, (unsigned)W)) fail(PLBM_ERR_IO, "cannot write " + path);
        }
    }

    // The host arrays take the newest results: copied from res_d, unless a step already wrote them.
    void copy_results()
    {
        wait_host();
        if (!host_results_newer.load())
            for (int i = 0; i < 4; ++i)
                cuda_check(cudaMemcpyAsync(res_h[i], res_d[i], nres * sizeof(double), cudaMemcpyDeviceToHost, stream),
                           "D2H results");
        cuda_check(cudaStreamSynchronize(stream), "results copy");
    }

    // res_d takes the newest results back from the host arrays where a step wrote those instead.
    void device_results_current()
    {
        if (!host_results_newer.load()) return;
        wait_host();
        for (int i = 0; i < 4; ++i)
            cuda_check(cudaMemcpyAsync(res_d[i], res_h[i], nres * sizeof(double), cudaMemcpyHostToDevice, stream),
                       "H2D results");
        cuda_check(cudaStreamSynchronize(stream), "results copy");
        host_results_newer = false;
    }

    // The per-step loop of the drivers (nptl.hpp:121-139): stop when paused or finished; results
    // go to the host on frame steps and after the final step.  Steps and frame copies are
    // enqueued without waiting; the host synchronises after about 5 ms of device work (at least
    // 32 steps), at the end, on pause and before writing an exported frame, then checks the status
    // word and publishes iteration, progress and the time per step.
    void loop()
    {
        try {
            const PhaseTrace run_trace("run");
            cuda_check(cudaSetDevice(opt.device), "cudaSetDevice");
            const unsigned T = props.time_steps, F = props.frame_update_interval;
            unsigned t = iteration.load(), done = t, max_pending = 32;
            auto c0 = std::chrono::steady_clock::now();
            auto publish = [&](unsigned upto) {
                cuda_check(cudaStreamSynchronize(stream), "step");
                check_status();
                const auto c1 = std::chrono::steady_clock::now();
                if (upto > done) frametime = std::chrono::duration<double, std::milli>(c1 - c0).count() / (double)(upto - done);
                c0 = c1;
                done = upto;
                iteration = upto;
                progress = (double)upto / (double)T;
                const double per_step = frametime.load();
                max_pending = per_step > 0 ? (unsigned)std::min(4096.0, std::max(32.0, 5.0 / per_step)) : 32u;
            };
            while (!stop.load() && t < T) {
                unsigned frame = t + (F - 1 - t % F);
                if (frame > T - 1) frame = T - 1;
                unsigned end;
                if (opt.use_graph && !export_fields && !debug && F >= 2 && F <= 256 && t % F == 0 && t + F < T) {
                    // a whole frame: one graph launch (its steps, results written to the host)
                    cuda_check(cudaGraphLaunch(frame_graph(t, F), stream), "frame graph launch");
                    host_results_newer = true;
                    end = t + F;
                } else if (t < frame) {
                    const unsigned chunk = std::max<unsigned>(graph_steps ? graph_steps : 32, 32);
                    end = std::min(frame, t + chunk);
                    run_plain(t, end);
                } else {
                    // a frame step writes its observables into the mapped host arrays itself (no
                    // copy after it; a reader of the reference's unsynchronised getters sees the
                    // arrays refreshed while the step runs)
                    wait_host();
                    cuda_check(launch_step(t, true, true), "step");
                    host_results_newer = true;
                    end = t + 1;
                    if (export_fields) {
                        publish(end);
                        export_frame(end);
                    }
                }
                t = end;
                if (t - done >= max_pending) publish(t);
            }
            if (t != done) publish(t);
            run_trace("steps and results done");
        } catch (const Status &s) {
            std::lock_guard<std::mutex> g(mu);
            worker_status = s.code;
            worker_error = s.msg;
        }
    }
};

namespace {

int set_err(plbm_handler *h, const Status &s)
{
    if (h) h->last_error = s.msg;
    else {
        std::lock_guard<std::mutex> g(g_create_mu);
        g_create_error = s.msg;
    }
    return s.code;
}

template <typename F>
int guarded(plbm_handler *h, F &&f)
{
    try {
        f();
        return PLBM_OK;
    } catch (const Status &s) {
        return set_err(h, s);
    } catch (const std::exception &e) {
        return set_err(h, Status{ PLBM_ERR_ARGUMENT, e.what() });
    }
}

}  // namespace

int plbm::max_threads_for(int alg, int prec, int lay)
{
    (void)alg; (void)lay;
    return prec == PLBM_F64_STRICT || prec == PLBM_F32_REF || prec == PLBM_F64_Q60 ? 256 : 512;
}

extern "C" {

void plbm_default_options(plbm_options *o)
{
    o->precision = PLBM_F64_STRICT;
    o->nan_protection = 1;
    o->use_graph = 1;
    o->device = 0;
    o->mask = nullptr;
    o->gather = PLBM_GATHER_AUTO;
}

int plbm_gather_form(plbm_handler *h, int *form)
{
    return guarded(h, [&] {
        if (!form) fail(PLBM_ERR_ARGUMENT, "form is NULL");
        *form = h->porous ? PLBM_GATHER_POROUS : PLBM_GATHER_OPEN;
    });
}

int plbm_validate(const plbm_properties *props)
{
    return guarded(nullptr, [&] {
        if (!props) fail(PLBM_ERR_ARGUMENT, "props is NULL");
        Props::make(*props).validate();
    });
}

static int create_common(plbm_handler *h, const plbm_options *opt, plbm_handler **out)
{
    if (opt) h->opt = *opt;
    else plbm_default_options(&h->opt);
    if (h->opt.gather < PLBM_GATHER_AUTO || h->opt.gather > PLBM_GATHER_POROUS) {
        set_err(nullptr, Status{ PLBM_ERR_ARGUMENT, "gather must be PLBM_GATHER_AUTO, PLBM_GATHER_OPEN or PLBM_GATHER_POROUS" });
        delete h;
        return PLBM_ERR_ARGUMENT;
    }
    // A settings file's "gb300" object chooses the precision unless the caller's options name
    // one other than the drop-in default.
    h->opt_precision_set = opt && (!h->from_json || opt->precision != PLBM_F64_STRICT);
    try {
        if (h->opt.mask) {
            Props p = h->from_json ? json_to_props(h->settings_path, 0, nullptr) : h->props;
            const size_t n = (size_t)(p.horizontal_nodes - 2) * (p.vertical_nodes - 2);
            h->mask_n = n;
            h->has_mask = true;
            h->mask_src = h->opt.mask;                             // valid during this call only
            h->opt.mask = nullptr;
        }
        h->build();
        h->mask_src = nullptr;
    } catch (const Status &s) {
        set_err(nullptr, s);
        delete h;
        return s.code;
    }
    *out = h;
    return PLBM_OK;
}

int plbm_create(const plbm_properties *props, const plbm_options *opt, plbm_handler **out)
{
    if (!props || !out) return set_err(nullptr, Status{ PLBM_ERR_ARGUMENT, "NULL argument" });
    auto *h = new plbm_handler();
    h->props = Props::make(*props);
    return create_common(h, opt, out);
}

int plbm_create_from_json(const char *settings_path, const plbm_options *opt, plbm_handler **out)
{
    if (!settings_path || !out) return set_err(nullptr, Status{ PLBM_ERR_ARGUMENT, "NULL argument" });
    auto *h = new plbm_handler();
    h->from_json = true;
    h->settings_path = settings_path;
    return create_common(h, opt, out);
}

void plbm_destroy(plbm_handler *h) { delete h; }

int plbm_initialize(plbm_handler *h)
{
    return guarded(h, [&] { h->build(); });
}

int plbm_start(plbm_handler *h)
{
    return guarded(h, [&] {
        if (h->active) return;   // SYCLAlgorithmHandler::start :378-386
        if (h->worker.joinable()) h->worker.join();
        h->stop = false;
        h->future_valid = true;
        h->worker = std::thread([h] { h->loop(); });
        h->active = true;
    });
}

int plbm_pause(plbm_handler *h)
{
    return guarded(h, [&] {
        h->stop = true;   // Control::forbid_execution; the step in flight completes
        if (h->worker.joinable()) h->worker.join();
        h->active = false;
    });
}

int plbm_block_until_finished(plbm_handler *h)
{
    return guarded(h, [&] {
        if (!h->future_valid)
            fail(PLBM_ERR_WAIT, "A thread accessed a blocking statement causing it to wait for an algorithm that has "
                                "not been launched.");
        if (h->worker.joinable()) h->worker.join();
        h->future_valid = false;
        h->active = false;
        std::lock_guard<std::mutex> g(h->mu);
        if (h->worker_status != PLBM_OK) {
            const Status s{ h->worker_status, h->worker_error };
            h->worker_status = PLBM_OK;
            throw s;
        }
    });
}

int plbm_is_finished(plbm_handler *h, int *finished)
{
    *finished = h->iteration.load() == h->props.time_steps;
    return PLBM_OK;
}

int plbm_get_results(plbm_handler *h, int which, const double **data, size_t *count)
{
    if (which < 0 || which > 3) return set_err(h, Status{ PLBM_ERR_ARGUMENT, "which must be 0..3" });
    return guarded(h, [&] {
        h->wait_host();
        *data = h->res_h[which];
        *count = h->nres;
    });
}

int plbm_get_extents(plbm_handler *h, unsigned *hn, unsigned *vn)
{
    *hn = h->props.horizontal_nodes;
    *vn = h->props.vertical_nodes;
    return PLBM_OK;
}

int plbm_get_domain(plbm_handler *h, unsigned out7[7])
{
    const Domain &d = h->dom;
    const unsigned v[7] = { d.total_node_count, d.horizontal_nodes, d.vertical_nodes, d.subdomain_vertical_nodes,
                            d.subdomain_horizontal_nodes, d.subdomain_count_vertical, d.subdomain_count_horizontal };
    std::memcpy(out7, v, sizeof v);
    return PLBM_OK;
}

int plbm_get_progress(plbm_handler *h, double *p) { *p = h->progress.load(); return PLBM_OK; }
int plbm_get_last_frametime(plbm_handler *h, double *ms) { *ms = h->frametime.load(); return PLBM_OK; }
int plbm_get_current_iteration(plbm_handler *h, unsigned *it) { *it = h->iteration.load(); return PLBM_OK; }

int plbm_get_properties(plbm_handler *h, plbm_properties *out)
{
    *out = h->props.to_c();
    return PLBM_OK;
}

int plbm_properties_to_json(const plbm_properties *props, const char *path)
{
    return guarded(nullptr, [&] {
        const Props p = Props::make(*props);
        props_to_json(p, props->vertical_nodes, props->horizontal_nodes, path);
    });
}

int plbm_json_to_properties(const char *path, int offset, plbm_properties *out)
{
    return guarded(nullptr, [&] {
        static thread_local Props keep;
        keep = json_to_props(path, offset, nullptr);
        *out = keep.to_c();
    });
}

int plbm_compute_domain(const plbm_properties *props, unsigned out7[7])
{
    return guarded(nullptr, [&] {
        const Props p = Props::make(*props);
        Domain d{};
        if (!make_domain(p, d)) fail(PLBM_ERR_PROPERTY, "work-group size below the swap algorithm's minimum of 6");
        const unsigned v[7] = { d.total_node_count, d.horizontal_nodes, d.vertical_nodes, d.subdomain_vertical_nodes,
                                d.subdomain_horizontal_nodes, d.subdomain_count_vertical, d.subdomain_count_horizontal };
        std::memcpy(out7, v, sizeof v);
    });
}

int plbm_make_flags(const plbm_properties *props, int8_t *out)
{
    return guarded(nullptr, [&] {
        const Props p = Props::make(*props);
        if (p.vertical_nodes < 4 || p.horizontal_nodes < 4) fail(PLBM_ERR_PROPERTY, "inner extents must be >= 2");
        const std::vector<int8_t> f = make_flags(p, nullptr);
        std::memcpy(out, f.data(), f.size());
    });
}

int plbm_run_steps(plbm_handler *h, unsigned n, double *ms_per_step)
{
    return guarded(h, [&] {
        if (h->worker.joinable()) fail(PLBM_ERR_ARGUMENT, "plbm_run_steps while the step loop runs");
        if (n == 0) return;
        const unsigned t0 = h->iteration.load();
        cuda_check(cudaSetDevice(h->opt.device), "cudaSetDevice");
        if (h->opt.use_graph) h->ensure_graph();
        cuda_check(cudaEventRecord(h->ev0, h->stream), "event");
        h->run_plain(t0, t0 + n - 1);
        cuda_check(h->launch_step(t0 + n - 1, true), "step");
        h->host_results_newer = false;
        cuda_check(cudaEventRecord(h->ev1, h->stream), "event");
        cuda_check(cudaEventSynchronize(h->ev1), "steps");
        float ms = 0;
        cuda_check(cudaEventElapsedTime(&ms, h->ev0, h->ev1), "elapsed");
        if (ms_per_step) *ms_per_step = ms / n;
        h->check_status();
        h->iteration = t0 + n;
        h->progress = (double)(t0 + n) / (double)h->props.time_steps;
    });
}

// Re-encodes the state of a handler that is not stepping into another shifted storage form and
// continues in it: the lattices (and npol's halo snapshots) hold the deviation from the same
// reference state in every shifted form, so each value is decoded, rescaled by a power of two and
// rounded once into the new form; the form's FP32 constants are rebuilt and the captured CUDA graphs
// dropped.  A state that does not fit the new form (F16C) leaves the handler unchanged.
int plbm_set_precision(plbm_handler *h, int precision)
{
    return guarded(h, [&] {
        auto shifted = [](int p) { return p == PLBM_F32 || p == PLBM_F16S || p == PLBM_BF16S || p == PLBM_F16C; };
        if (h->worker.joinable()) fail(PLBM_ERR_ARGUMENT, "plbm_set_precision while the step loop runs");
        if (!shifted(h->prec) || !shifted(precision))
            fail(PLBM_ERR_ARGUMENT, "plbm_set_precision converts between the shifted forms PLBM_F32, PLBM_F16S, "
                                    "PLBM_BF16S and PLBM_F16C");
        if (precision == h->prec) return;
        cuda_check(cudaSetDevice(h->opt.device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(h->stream), "pending work");
        plbm::StepParams b = h->base;
        plbm::fill_float_constants(b, true, h->two_lattice(), h->props.irho, h->props.orho,
                                   precision == PLBM_F16S ? (double)plbm::F16_SCALE : 1.0);
        if (precision == PLBM_F16C) {
            double worst = 0;
            for (int d = 0; d < 9; ++d)
                worst = std::max({ worst, std::fabs((double)b.weightf[d]), std::fabs((double)b.feq_inf[d]),
                                   std::fabs((double)b.feq_outf[d]),
                                   std::fabs((double)b.weightf[d] + (double)b.shift_wg[d] * (h->W - 1)) });
            if (!(worst < 0.5))
                fail(PLBM_ERR_NUMERIC, "f16c stores deviations |f - w rho0| < 0.5; these boundary densities exceed it");
        }
        const size_t eb = storage_bytes(precision);
        const int nl = h->two_lattice() ? 2 : 1;
        void *nlat[2] = { nullptr, nullptr }, *nhalo[2] = { nullptr, nullptr };
        const size_t hn = h->alg == 2 ? std::max<size_t>(b.halo_elems, 1) : 0;
        auto release_new = [&] {
            for (auto &q : nlat) { if (q) cudaFree(q); q = nullptr; }
            for (auto &q : nhalo) { if (q) cudaFree(q); q = nullptr; }
        };
        try {
            cuda_check(cudaMemsetAsync(h->status_d, 0, sizeof(int), h->stream), "memset status");
            for (int i = 0; i < nl; ++i) {
                cuda_check(cudaMalloc(&nlat[i], 9ull * h->N * eb), "cudaMalloc lattice");
                cuda_check(plbm::launch_convert_shifted(h->lat[i], h->prec, nlat[i], precision, 9ull * h->N, h->status_d,
                                                        h->stream), "lattice conversion");
            }
            for (int i = 0; i < 2 && hn; ++i) {
                cuda_check(cudaMalloc(&nhalo[i], hn * eb), "cudaMalloc halo");
                cuda_check(plbm::launch_convert_shifted(h->halo[i], h->prec, nhalo[i], precision, b.halo_elems,
                                                        h->status_d, h->stream), "halo conversion");
            }
            int st = 0;
            cuda_check(cudaMemcpyAsync(&st, h->status_d, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "status");
            cuda_check(cudaStreamSynchronize(h->stream), "conversion");
            if (st) fail(PLBM_ERR_NUMERIC, "the state does not fit the new storage form (f16c: |f - w rho0| < 0.5)");
        } catch (...) {
            release_new();
            throw;
        }
        for (int i = 0; i < nl; ++i) { cudaFree(h->lat[i]); h->lat[i] = nlat[i]; nlat[i] = nullptr; }
        for (int i = 0; i < 2 && hn; ++i) { cudaFree(h->halo[i]); h->halo[i] = nhalo[i]; nhalo[i] = nullptr; }
        h->base = b;
        h->prec = precision;
        if (h->gexec) cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
        h->graph_steps = 0;
        for (auto &f : h->frame_gexec) { if (f) cudaGraphExecDestroy(f); f = nullptr; }
        h->frame_graph_len = 0;
    });
}

int plbm_run_to_residual(plbm_handler *h, double target, unsigned K, unsigned max_steps, unsigned *steps,
                         double *residual)
{
    return guarded(h, [&] {
        if (K == 0) fail(PLBM_ERR_ARGUMENT, "K must be >= 1");
        if (!h->jprev_d) {
            cuda_check(cudaMalloc(&h->jprev_d, 2 * h->nres * sizeof(double)), "cudaMalloc residual");
            cuda_check(cudaMemsetAsync(h->jprev_d, 0, 2 * h->nres * sizeof(double), h->stream), "memset");
        }
        unsigned done = 0;
        double r = INFINITY;
        while (done < max_steps) {
            const unsigned n = std::min(K, max_steps - done);
            const long long before = (long long)h->iteration.load();
            double ms = 0;
            const int rc = plbm_run_steps(h, n, &ms);
            if (rc != PLBM_OK) throw Status{ rc, h->last_error };
            done += n;
            double sums[2] = { 0, 0 };
            cuda_check(plbm::launch_residual(h->res_d[1], h->res_d[2], h->jprev_d, h->jprev_d + h->nres, h->flags_d,
                                             h->nres, h->red_d, h->stream), "residual");
            cuda_check(cudaMemcpyAsync(sums, h->red_d, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H");
            cuda_check(cudaStreamSynchronize(h->stream), "residual");
            // a residual needs the snapshot of exactly K steps earlier (possibly from the previous call)
            if (n == K && h->jprev_iter == before)
                r = sums[1] > 0 ? std::sqrt(sums[0]) / ((double)K * std::sqrt(sums[1])) : INFINITY;
            h->jprev_iter = (long long)h->iteration.load();
            if (r < target) break;
        }
        h->copy_results();
        *steps = done;
        *residual = r;
    });
}

int plbm_porous_disks(unsigned inner_w, unsigned inner_h, uint64_t seed, double porosity, double rmin, double rmax,
                      int8_t *out)
{
    int count = 0;
    const int rc = guarded(nullptr, [&] {
        if (inner_w < 2 || inner_h < 3 || !(porosity > 0 && porosity <= 1) || !(rmin > 0 && rmax >= rmin))
            fail(PLBM_ERR_ARGUMENT, "invalid porous-disk parameters");
        const int W = (int)inner_w, H = (int)inner_h;
        std::vector<int8_t> m((size_t)W * H, 0);
        for (int x = 0; x < W; ++x) { m[x] = 1; m[(size_t)(H - 1) * W + x] = 1; }
        // splitmix64 stream
        uint64_t st = seed;
        auto next = [&st]() {
            uint64_t z = (st += 0x9E3779B97F4A7C15ull);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            return z ^ (z >> 31);
        };
        auto uni = [&]() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); };
        // spatial hash of placed disks on cells of 2*rmax
        const double cell = 2 * rmax;
        const int gx = (int)(W / cell) + 1, gy = (int)(H / cell) + 1;
        std::vector<std::vector<int>> grid((size_t)gx * gy);
        std::vector<double> cx, cy, cr;
        const double interior = (double)W * (H - 2);
        double solid = 0;
        const double target = (1 - porosity) * interior;
        long attempts = 0;
        const long max_attempts = 200 * (long)(interior / (3.14159 * rmin * rmin) + 10);
        while (solid < target && attempts < max_attempts) {
            ++attempts;
            const double r = rmin + (rmax - rmin) * uni();
            const double x = uni() * W, y = 1 + r + uni() * (H - 2 - 2 * r);
            const int ix = (int)(x / cell), iy = (int)(y / cell);
            bool ok = true;
            for (int ny = std::max(0, iy - 1); ny <= std::min(gy - 1, iy + 1) && ok; ++ny)
                for (int nx = std::max(0, ix - 1); nx <= std::min(gx - 1, ix + 1) && ok; ++nx)
                    for (int k : grid[(size_t)ny * gx + nx]) {
                        const double dx = cx[k] - x, dy = cy[k] - y, rr = cr[k] + r + 1;
                        if (dx * dx + dy * dy < rr * rr) { ok = false; break; }
                    }
            if (!ok) continue;
            const int k = (int)cx.size();
            cx.push_back(x); cy.push_back(y); cr.push_back(r);
            grid[(size_t)iy * gx + ix].push_back(k);
            for (int py = std::max(1, (int)(y - r)); py <= std::min(H - 2, (int)(y + r) + 1); ++py)
                for (int px = std::max(0, (int)(x - r)); px <= std::min(W - 1, (int)(x + r) + 1); ++px) {
                    const double dx = px + 0.5 - x, dy = py + 0.5 - y;
                    int8_t &c = m[(size_t)py * W + px];
                    if (c == 0 && dx * dx + dy * dy <= r * r) { c = 1; solid += 1; }
                }
        }
        std::memcpy(out, m.data(), m.size());
        count = (int)cx.size();
    });
    return rc == PLBM_OK ? count : rc;
}

int plbm_set_equilibrium(plbm_handler *h, const double *rho, const double *jx, const double *jy)
{
    return guarded(h, [&] {
        if (h->alg != 0 && h->alg != 1) fail(PLBM_ERR_ARGUMENT, "plbm_set_equilibrium supports nptl and lptl");
        if (h->worker.joinable()) fail(PLBM_ERR_ARGUMENT, "plbm_set_equilibrium while the step loop runs");
        const unsigned par = h->iteration.load() & 1u;
        double *tmp = nullptr;
        cuda_check(cudaMalloc(&tmp, 3 * h->nres * sizeof(double)), "cudaMalloc fields");
        std::unique_ptr<double, decltype(&cudaFree)> keep(tmp, &cudaFree);
        const double *src[3] = { rho, jx, jy };
        for (int i = 0; i < 3; ++i)
            cuda_check(cudaMemcpyAsync(tmp + i * h->nres, src[i], h->nres * sizeof(double), cudaMemcpyHostToDevice,
                                       h->stream), "H2D fields");
        cuda_check(plbm::launch_set_equilibrium(h->lat[par], h->prec, h->lay, h->base, tmp, tmp + h->nres,
                                                tmp + 2 * h->nres, h->stream), "equilibrium");
        // the outlet reads the previous step's jy of column x' = W-2; steps never write it for a
        // solid node there, so those entries keep the zero a rest start holds
        if (h->W < 2) { cuda_check(cudaStreamSynchronize(h->stream), "equilibrium"); h->jprev_iter = -1; return; }
        std::vector<int8_t> solid(h->H);
        cuda_check(cudaMemcpy2DAsync(solid.data(), 1, h->flags_d + (h->W - 2), h->W, 1, h->H, cudaMemcpyDeviceToHost,
                                     h->stream), "D2H flags");
        cuda_check(cudaStreamSynchronize(h->stream), "flags");
        std::vector<double> col(h->H);
        for (int y = 0; y < h->H; ++y) col[y] = solid[y] ? 0.0 : jy[(size_t)y * h->W + h->W - 2];
        cuda_check(cudaMemcpyAsync(h->jy_d + (size_t)par * h->H, col.data(), h->H * sizeof(double),
                                   cudaMemcpyHostToDevice, h->stream), "H2D jy");
        cuda_check(cudaStreamSynchronize(h->stream), "equilibrium");
        h->jprev_iter = -1;
    });
}

int plbm_set_frame_export(plbm_handler *h, const char *directory, unsigned fields)
{
    return guarded(h, [&] {
        if (h->worker.joinable()) fail(PLBM_ERR_ARGUMENT, "plbm_set_frame_export while the step loop runs");
        if (!directory || !*directory || fields == 0) {
            h->export_dir.clear();
            h->export_fields = 0;
            return;
        }
        if (fields > 15u) fail(PLBM_ERR_ARGUMENT, "fields: bits 0..3 (density, x/y momentum, |momentum|)");
        std::error_code ec;
        std::filesystem::create_directories(directory, ec);
        if (ec || !std::filesystem::is_directory(directory))
            fail(PLBM_ERR_IO, std::string("cannot create export directory ") + directory);
        h->export_dir = directory;
        h->export_fields = fields;
    });
}

int plbm_write_npy(const char *path, const double *data, unsigned rows, unsigned cols)
{
    if (!path || (!data && rows != 0 && cols != 0)) return PLBM_ERR_ARGUMENT;
    return write_npy(path, data, rows, cols) ? PLBM_OK : PLBM_ERR_IO;
}

int plbm_sync_results(plbm_handler *h)
{
    return guarded(h, [&] { h->copy_results(); });
}

int plbm_launches_per_step(plbm_handler *h, unsigned *n)
{
    *n = h->debug ? 3 : 1;
    return PLBM_OK;
}

int plbm_bytes_per_node(plbm_handler *h, double *bytes)
{
    *bytes = 18.0 * (double)storage_bytes(h->prec);
    return PLBM_OK;
}

int plbm_mass_momentum(plbm_handler *h, double out3[3])
{
    return guarded(h, [&] {
        h->device_results_current();
        cuda_check(plbm::launch_reduce_results(h->res_d[0], h->res_d[1], h->res_d[2], h->flags_d, h->nres, h->red_d,
                                               h->stream),
                   "reduce");
        cuda_check(cudaMemcpyAsync(out3, h->red_d, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H");
        cuda_check(cudaStreamSynchronize(h->stream), "reduce");
    });
}

const char *plbm_last_error(const plbm_handler *h)
{
    if (h) return h->last_error.c_str();
    std::lock_guard<std::mutex> g(g_create_mu);
    g_tls_error = g_create_error;
    return g_tls_error.c_str();
}

const char *plbm_version(void)
{
    return plbm::CHECKED_BUILD ? "portlbm_gb300 0.2 (sm_103a, checked)" : "portlbm_gb300 0.2 (sm_103a)";
}

}  // extern "C"
