/* CPU restatement of the reference's coupled LB/DEM step.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle: tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it to check
 * or to time against; the product (liblbdem.so) never links or calls it.
 *
 * It restates the reference's algorithm serially, on dense arrays, in the
 * reference's own operation order (see the file:line citations in
 * lbdem_oracle.cpp), including its defined-behaviour pins and its quirks.
 * Its output is pinned against the compiled reference (oracle/ref_driver.cpp):
 * tests/test_oracle_golden.py compares it bit for bit with the per-step
 * hashes of the reference's state that tests/golden/make_golden.py recorded.
 */
#ifndef LBDEM_ORACLE_H
#define LBDEM_ORACLE_H
#include "../include/lbdem.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

int oracle_create(const lbdem_config* cfg, oracle_ctx** out);
void oracle_destroy(oracle_ctx* ctx);
const char* oracle_last_error(const oracle_ctx* ctx);
int oracle_dem_step(oracle_ctx* ctx);
int oracle_coupling_step(oracle_ctx* ctx);
int oracle_lb_step(oracle_ctx* ctx);
int oracle_free_surface_step(oracle_ctx* ctx);
/* n x goCycle (src/main.cpp:38-67), no IO */
int oracle_cycle(oracle_ctx* ctx, int32_t n);
/* write the same dump layout as oracle/ref_driver.cpp */
int oracle_dump(oracle_ctx* ctx, const char* path);
/* counters: [0] goCycle count, [1] demTimeStep, [2] neighbour rebuilds,
 * [3] active nodes, [4] interface nodes */
int oracle_counters(oracle_ctx* ctx, int64_t* out5);
double oracle_dem_time(oracle_ctx* ctx);
/* OpenMP threads of the per-node loops (reconstruction, collision); the
 * results do not depend on it (every node is updated on its own) */
int oracle_set_threads(int32_t n);
int oracle_max_threads(void);
/* impactor 0 position/velocity, 6 doubles */
int oracle_object0(oracle_ctx* ctx, double* out6);

#ifdef __cplusplus
}
#endif
#endif
