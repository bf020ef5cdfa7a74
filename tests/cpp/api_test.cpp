// C++ API test of the drop-in header, in the shape of the reference's own tests:
//   smoke      tests/smoke_test.cpp:40-97   (lptl + stream, 126x30, tau 0.6, rho_in 1.3, 100 steps)
//   regression tests/test_regression.cpp:67-181 (lptl + stream Hagen-Poiseuille 30x14, tau 1.0,
//              rho 1.01 / 1.0, 8000 steps: parabolic profile checks)
//   errors     validate() / unknown algorithm / block_until_finished twice
//   interface  get_properties() / get_domain() through std::unique_ptr<AlgorithmHandler>
//              (algorithm_handler.hpp:146,151), checked against core::Domain(Properties&)
// Exit status 0 when every check holds.
#include "portlbm_gb300.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <numeric>

static int failures = 0;
#define CHECK(c)                                                                  \
    do {                                                                          \
        if (!(c)) { std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); ++failures; } \
    } while (0)

static void smoke()
{
    lbm::core::Properties props("lptl", "stream", false, 64, 100, 100, "Hagen-Poiseuille", 30, 126, 0.0, 0.0, 1.3,
                                0.0, 0.0, 1.0, 0.6);
    props.validate();
    auto handler = lbm::create_handler(props);
    handler->start();
    handler->block_until_finished();
    const auto &rho = handler->get_densities();
    const auto &jx = handler->get_x_velocities();
    CHECK(!rho.empty() && rho.size() == jx.size());
    CHECK(std::none_of(rho.begin(), rho.end(), [](double v) { return std::isnan(v); }));
    CHECK(std::accumulate(rho.begin(), rho.end(), 0.0) / rho.size() > 0.5);
    CHECK(std::any_of(jx.begin(), jx.end(), [](double v) { return std::abs(v) > 1e-12; }));
}

static void regression()
{
    lbm::core::Properties props("lptl", "stream", false, 16, 8000, 8000, "Hagen-Poiseuille", 14, 30, 0.0, 0.0, 1.01,
                                0.0, 0.0, 1.0, 1.0);
    auto handler = lbm::create_handler(props);
    handler->start();
    handler->block_until_finished();
    const unsigned w = handler->get_horizontal_nodes() - 2, h = handler->get_vertical_nodes() - 2;
    CHECK(w == 30 && h == 14);
    const auto &jx = handler->get_x_velocities();
    std::vector<double> prof(h);
    for (unsigned r = 0; r < h; ++r) prof[r] = jx[w / 2 + r * w];
    double umax = 0, sum = 0;
    unsigned peak = 0;
    for (unsigned r = 1; r + 1 < h; ++r) {
        CHECK(prof[r] > 0);
        if (prof[r] > umax) { umax = prof[r]; peak = r; }
        sum += prof[r];
    }
    for (unsigned i = 1; i <= h / 2; ++i) CHECK(std::abs(prof[i] - prof[h - 1 - i]) / umax < 0.01);
    const unsigned centre = (1 + h - 2) / 2;
    CHECK(peak + 1 >= centre && peak <= centre + 1);
    const double ratio = umax / (sum / (h - 2));
    CHECK(ratio > 1.35 && ratio < 1.55);
}

static void errors()
{
    bool thrown = false;
    try {
        lbm::core::Properties("nptl", "stream", false, 64, 10, 10, "cube", 30, 62, 0, 0, 1.1, 0, 0, 1.0, 0.6).validate();
    } catch (const lbm::exceptions::json::PropertyArgumentException &) {
        thrown = true;
    }
    CHECK(thrown);
    thrown = false;
    try {
        lbm::create_handler(lbm::core::Properties("abcd", "stream", false, 64, 10, 10, "circle", 30, 62, 0, 0, 1.1, 0,
                                                  0, 1.0, 0.6));
    } catch (const lbm::exceptions::Exception &) {
        thrown = true;
    }
    CHECK(thrown);
    auto handler = lbm::create_handler(
        lbm::core::Properties("nptl", "stream", false, 64, 10, 10, "circle", 30, 62, 0, 0, 1.1, 0, 0, 1.0, 0.6));
    handler->start();
    handler->block_until_finished();
    thrown = false;
    try {
        handler->block_until_finished();
    } catch (const lbm::exceptions::algorithm::WaitException &) {
        thrown = true;
    }
    CHECK(thrown);
    CHECK(handler->is_finished() && handler->get_current_iteration() == 10);
}

static void interface()
{
    const char *algs[4] = { "nptl", "lptl", "npol", "nsol" };
    for (const char *alg : algs) {
        lbm::core::Properties props(alg, "bundle", false, 64, 20, 20, "circle", 37, 91, 0.0, 0.0, 1.05, 0.0, 0.0, 1.0,
                                    0.7);
        std::unique_ptr<lbm::execution::AlgorithmHandler> handler = lbm::create_handler(props);
        const lbm::core::Properties &got = handler->get_properties();
        CHECK(got.algorithm == alg && got.data_layout == "bundle" && got.scenario == "circle");
        CHECK(got.vertical_nodes == 39 && got.horizontal_nodes == 93 && got.domain_node_count == 37u * 91u);
        CHECK(got.work_group_size == 64 && got.time_steps == 20 && got.relaxation_time == 0.7);
        CHECK(got.inlet_density == 1.05 && got.outlet_density == 1.0);
        const lbm::core::Domain &dom = handler->get_domain();
        const lbm::core::Domain want(props);
        CHECK(dom.total_node_count == want.total_node_count && dom.horizontal_nodes == want.horizontal_nodes &&
              dom.vertical_nodes == want.vertical_nodes);
        CHECK(dom.subdomain_vertical_nodes == want.subdomain_vertical_nodes &&
              dom.subdomain_horizontal_nodes == want.subdomain_horizontal_nodes &&
              dom.subdomain_count_vertical == want.subdomain_count_vertical &&
              dom.subdomain_count_horizontal == want.subdomain_count_horizontal);
        CHECK(dom.total_node_count >= 39u * 93u);
        CHECK(handler->processing_element_constraint == 1024);
        handler->start();
        handler->block_until_finished();
        CHECK(handler->get_current_iteration() == 20 && handler->get_densities().size() == 37u * 91u);
    }
}

int main()
{
    interface();
    smoke();
    regression();
    errors();
    std::printf("%s (%d failures)\n", failures ? "FAILED" : "OK", failures);
    return failures ? 1 : 0;
}
