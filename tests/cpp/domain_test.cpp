// core::Domain(Properties&) of the drop-in header, without a GPU: prints the seven fields for
// each algorithm, inner extents and work-group size given on the command line
// (domain_test W H WG), one line per algorithm; exits 2 unless nsol with a work-group size below
// 6 throws PropertyArgumentException as the reference's swap set-up does
// (src/lbm/core/simulation.cpp:329-353).
#include "portlbm_gb300.hpp"

#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv)
{
    if (argc != 4) return 1;
    const unsigned w = (unsigned)std::atoi(argv[1]), h = (unsigned)std::atoi(argv[2]), wg = (unsigned)std::atoi(argv[3]);
    const char *algs[4] = { "nptl", "lptl", "npol", "nsol" };
    for (const char *a : algs) {
        lbm::core::Properties p(a, "stream", false, wg, 10, 10, "circle", h, w, 0, 0, 1.05, 0, 0, 1.0, 0.7);
        const lbm::core::Domain d(p);
        std::printf("%s %u %u %u %u %u %u %u\n", a, d.total_node_count, d.horizontal_nodes, d.vertical_nodes,
                    d.subdomain_vertical_nodes, d.subdomain_horizontal_nodes, d.subdomain_count_vertical,
                    d.subdomain_count_horizontal);
    }
    try {
        lbm::core::Properties p("nsol", "stream", false, 4, 10, 10, "circle", h, w, 0, 0, 1.05, 0, 0, 1.0, 0.7);
        const lbm::core::Domain d(p);
    } catch (const lbm::exceptions::json::PropertyArgumentException &) {
        return 0;
    }
    return 2;
}
