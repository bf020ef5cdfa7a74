// C++ API test of the drop-in header, in the shape of the reference's own tests:
//   smoke      tests/smoke_test.cpp:40-97   (lptl + stream, 126x30, tau 0.6, rho_in 1.3, 100 steps)
//   regression tests/test_regression.cpp:67-181 (lptl + stream Hagen-Poiseuille 30x14, tau 1.0,
//              rho 1.01 / 1.0, 8000 steps: parabolic profile checks)
//   errors     validate() / unknown algorithm / block_until_finished twice
// Exit status 0 when every check holds.
#include "portlbm_gb300.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
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

int main()
{
    smoke();
    regression();
    errors();
    std::printf("%s (%d failures)\n", failures ? "FAILED" : "OK", failures);
    return failures ? 1 : 0;
}
