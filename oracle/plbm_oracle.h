/*
 * plbm_oracle.h — CPU restatement of PortLBM's per-timestep D2Q9 BGK update.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA path is checked
 * against; it is never linked into, loaded by, or called from the product
 * library (portlbm_gb300/csrc).  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may use it.
 *
 * Every function restates one piece of the reference (SC-SGS/PortLBM) literally,
 * including its unsigned index arithmetic and boundary quirks, and cites the
 * reference file:line it follows.  Arithmetic is IEEE double, compiled with
 * -ffp-contract=off so that the operation order below is the one executed.
 */
#ifndef PLBM_ORACLE_H
#define PLBM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { PLBMO_NPTL = 0, PLBMO_LPTL = 1, PLBMO_NPOL = 2, PLBMO_NSOL = 3 };
enum { PLBMO_COLLISION = 0, PLBMO_STREAM = 1, PLBMO_BUNDLE = 2 };
enum {
    PLBMO_HAGEN_POISEUILLE = 0, PLBMO_WALLS = 1, PLBMO_CIRCLE = 2, PLBMO_SQUARE = 3,
    PLBMO_WING = 4, PLBMO_SKYSCRAPER = 5, PLBMO_POROUS = 6, PLBMO_PLATE = 7,
    PLBMO_CUSTOM = 100
};

/* Mirrors core::Domain (include/lbm/core/domain.hpp:29-85). */
typedef struct {
    unsigned total_node_count, horizontal_nodes, vertical_nodes;
    unsigned subdomain_vertical_nodes, subdomain_horizontal_nodes;
    unsigned subdomain_count_vertical, subdomain_count_horizontal;
} plbmo_domain;

typedef struct plbmo_sim plbmo_sim;

/* Domain arithmetic for one algorithm; X,V are stored extents (inner + 2).
 * Returns 0, or -1 when nsol's work-group size is below 6. */
int plbmo_domain_for(int algorithm, unsigned work_group_size, unsigned X, unsigned V, plbmo_domain *out);

/* glibc random()/rand() TYPE_3 additive-feedback generator restated; state starts from seed 1
 * as an unseeded process does.  Exposed for tests. */
void plbmo_rand_reset(unsigned seed);
int plbmo_rand(void);

/* Creates a simulation.  inner_w/inner_h are settings horizontalNodes/verticalNodes.
 * custom_mask (scenario PLBMO_CUSTOM only): inner_w*inner_h int8 flags (0 fluid, 1 solid),
 * row-major from (x=1,y=1); it replaces walls and stencil entirely.
 * Returns NULL on an illegal configuration. */
plbmo_sim *plbmo_create(int algorithm, int layout, unsigned work_group_size, int scenario,
                        unsigned inner_w, unsigned inner_h,
                        double inlet_vx, double inlet_vy, double inlet_density,
                        double outlet_vx, double outlet_vy, double outlet_density,
                        double relaxation_time, int nan_protection, const int8_t *custom_mask);
void plbmo_destroy(plbmo_sim *s);
/* Advances n timesteps (emplace -> outlet -> stream/collide [-> swap] per step). */
void plbmo_run(plbmo_sim *s, unsigned steps);
/* Copies the (inner_w*inner_h) result arrays: which = 0 rho, 1 jx, 2 jy, 3 |j|. */
void plbmo_results(const plbmo_sim *s, int which, double *out);
/* Copies the flag grid of the expanded domain (total_node_count int8). */
void plbmo_flags(const plbmo_sim *s, int8_t *out);
/* Copies lattice `which` (0/1) as stored (9*total_node_count doubles); returns count or 0. */
size_t plbmo_lattice(const plbmo_sim *s, int which, double *out);
void plbmo_get_domain(const plbmo_sim *s, plbmo_domain *out);
/* Threads used by plbmo_run (OpenMP); 1 when built without OpenMP. */
int plbmo_threads(void);

#ifdef __cplusplus
}
#endif
#endif
