/* ORACLE -- test infrastructure only.  C API of the CPU restatement of the
 * OllinAxis-BiB evolution path; it takes the same ollin_params as the GPU
 * library (include/ollin_gpu.h) so that one harness drives both. */
#ifndef OLLIN_ORACLE_H
#define OLLIN_ORACLE_H
#include "../include/ollin_gpu.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct ollin_oracle ollin_oracle;
const char* ollin_oracle_last_error(void);
int ollin_oracle_create(const ollin_params* p, ollin_oracle** out);
void ollin_oracle_destroy(ollin_oracle* o);
int ollin_oracle_initial_data(ollin_oracle* o);
int ollin_oracle_initialize(ollin_oracle* o);
int ollin_oracle_step(ollin_oracle* o, double* t_out);
int ollin_oracle_num_levels(const ollin_oracle* o);
int ollin_oracle_dims(const ollin_oracle* o, int level, int* nr, int* nz, int* ghost);
double ollin_oracle_time(const ollin_oracle* o, int level);
int ollin_oracle_get(ollin_oracle* o, int level, const char* name, double* a, int ld_r);
int ollin_oracle_set(ollin_oracle* o, int level, const char* name, const double* a, int ld_r);
int ollin_oracle_aux(ollin_oracle* o, int level);
int ollin_oracle_constraints(ollin_oracle* o, int level);
int ollin_oracle_maximal_slicing(ollin_oracle* o, const double* va_max);
int ollin_oracle_grid(const ollin_oracle* o, int gid, int* box, int* level);
int ollin_oracle_norms(ollin_oracle* o, int level, const char* name, double out[5]);
int ollin_oracle_interp(ollin_oracle* o, int level, const char* name, const double* rz, int n, double* out);
double ollin_oracle_point_updates(const ollin_oracle* o);
/* OpenMP threads of the oracle's loops from now on (>= 1), and the current
 * number; the CPU baselines time one and all host cores in one process */
void ollin_oracle_set_threads(int n);
int ollin_oracle_max_threads(void);
/* iteration counts of the last elliptic solve on this thread: steps[0] of
 * the coarse phase, steps[1] of the all-level phase (0 if there was none) */
int ollin_oracle_ell_stats(int steps[2], double* gres);
#ifdef __cplusplus
}
#endif
#endif
