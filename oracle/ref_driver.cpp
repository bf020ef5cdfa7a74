// ref_driver.cpp — TEST INFRASTRUCTURE.  A C entry point around the reference's own algorithm
// classes (SC-SGS/PortLBM include/lbm/gpu/{nptl,lptl,npol,nsol}/*.hpp, src/lbm/core/simulation.cpp),
// compiled from the reference tree against the host SYCL subset in oracle/ref_shim.  It is built
// into oracle/_ref/ (never committed, never shipped) and used only to pin the restated oracle and
// to generate tests/golden fixtures.
#include "lbm/core/constants.hpp"
#include "lbm/file_interaction/file_interaction.hpp"
#include "lbm/gpu/lptl/lptl.hpp"
#include "lbm/gpu/npol/npol.hpp"
#include "lbm/gpu/nptl/nptl.hpp"
#include "lbm/gpu/nsol/nsol.hpp"

#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

// The settings-file I/O (src/lbm/file_interaction/file_interaction.cpp) needs nlohmann/json, which
// is not available; simulation.cpp only reaches it on its self-correction paths, never exercised here.
void lbm::file_interaction::properties_to_json(const lbm::core::Properties &) {}
lbm::core::Properties lbm::file_interaction::json_to_properties(const std::string &, const int)
{
    throw std::runtime_error("settings I/O is not part of the oracle build");
}

namespace {

struct RefSim {
    sycl::queue q;
    std::unique_ptr<lbm::execution::SYCLAlgorithm> alg;
};

template <class A>
std::unique_ptr<lbm::execution::SYCLAlgorithm> make(int alg, sycl::queue &q, const lbm::core::Properties &p)
{
    switch (alg) {
    case 0: return std::make_unique<lbm::gpu::nptl::NPTL<A>>(q, p);
    case 1: return std::make_unique<lbm::gpu::lptl::LPTL<A>>(q, p);
    case 2: return std::make_unique<lbm::gpu::npol::NPOL<A>>(q, p);
    default: return std::make_unique<lbm::gpu::nsol::NSOL<A>>(q, p);
    }
}

}  // namespace

extern "C" {

// Builds the reference simulation for `time_steps` steps; scenario is one of the reference's names.
void *refo_create(int alg, int layout, unsigned wg, const char *scenario, unsigned inner_w, unsigned inner_h,
                  unsigned time_steps, double ivx, double ivy, double irho, double ovx, double ovy, double orho,
                  double tau, unsigned rand_seed)
{
    static const char *algs[] = { "nptl", "lptl", "npol", "nsol" };
    static const char *lays[] = { "collision", "stream", "bundle" };
    std::srand(rand_seed);
    lbm::core::Properties props(algs[alg], lays[layout], false, wg, time_steps, time_steps, scenario, inner_h, inner_w,
                                (lbm::real_type)ivx, (lbm::real_type)ivy, (lbm::real_type)irho, (lbm::real_type)ovx,
                                (lbm::real_type)ovy, (lbm::real_type)orho, (lbm::real_type)tau);
    auto *s = new RefSim();
    try {
        if (layout == 0) s->alg = make<lbm::core::access::CollisionAccessor>(alg, s->q, props);
        else if (layout == 1) s->alg = make<lbm::core::access::StreamAccessor>(alg, s->q, props);
        else s->alg = make<lbm::core::access::BundleAccessor>(alg, s->q, props);
    } catch (...) {
        delete s;
        return nullptr;
    }
    return s;
}

// Runs the reference's step loop (execute() on its worker thread) to the end.
void refo_run(void *h)
{
    auto *s = static_cast<RefSim *>(h);
    s->alg->simulation->control->allow_execution();
    s->alg->execute();
    s->alg->block_until_finished();
}

unsigned refo_result_count(void *h) { return (unsigned)static_cast<RefSim *>(h)->alg->simulation->results->densities_cpu->size(); }

void refo_results(void *h, int which, double *out)
{
    auto &r = *static_cast<RefSim *>(h)->alg->simulation->results;
    const std::vector<lbm::real_type> *v = which == 0 ? r.densities_cpu.get() : which == 1 ? r.x_velocities_cpu.get()
                                          : which == 2 ? r.y_velocities_cpu.get() : r.absolute_velocities_cpu.get();
    for (size_t i = 0; i < v->size(); ++i) out[i] = (double)(*v)[i];
}

void refo_domain(void *h, unsigned out7[7])
{
    const auto &d = *static_cast<RefSim *>(h)->alg->simulation->domain;
    const unsigned v[7] = { d.total_node_count, d.horizontal_nodes, d.vertical_nodes, d.subdomain_vertical_nodes,
                            d.subdomain_horizontal_nodes, d.subdomain_count_vertical, d.subdomain_count_horizontal };
    std::memcpy(out7, v, sizeof v);
}

void refo_flags(void *h, int8_t *out)
{
    const auto &sim = *static_cast<RefSim *>(h)->alg->simulation;
    std::memcpy(out, sim.data->phase_information, sim.domain->total_node_count);
}

void refo_destroy(void *h) { delete static_cast<RefSim *>(h); }

int refo_real_bytes(void) { return (int)sizeof(lbm::real_type); }

}  // extern "C"
