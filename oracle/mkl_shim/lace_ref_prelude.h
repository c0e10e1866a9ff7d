/*
 * Force-included (g++ -include) ahead of every LACE source compiled into the
 * CPU oracle (oracle/_ref).  Test infrastructure only.
 *
 * 1. LACE is built serially (no -fopenmp) so that the reference runs in
 *    its deterministic one-thread order (Gauss-Seidel order for ParILU and
 *    ParCSRTRSV, sequential reductions for FGMRES).  The handful of OpenMP
 *    runtime calls LACE makes are provided by the MKL stand-in library.
 * 2. LACE allocates through posix_memalign with up to 64 bytes of alignment
 *    padding beyond the requested size (include/dense_types.h:430-449), and
 *    its FGMRES reads one element past the last Krylov column when it forms
 *    the final reflector of a cycle (src/fgmres_householder_restart.cpp:477,
 *    481: n-search elements starting at row search+1).  The stand-in
 *    allocator zero-fills the padding so that read returns 0.0, the value the
 *    algorithm intends.
 */
#ifndef LACE_REF_PRELUDE_H
#define LACE_REF_PRELUDE_H

#include <stddef.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif
double omp_get_wtime(void);
int omp_get_num_threads(void);
int omp_get_max_threads(void);
int omp_get_num_procs(void);
int omp_get_thread_num(void);
void omp_set_num_threads(int n);
int lace_shim_posix_memalign(void **ptr, size_t alignment, size_t size);
#ifdef __cplusplus
}
#endif

#define posix_memalign lace_shim_posix_memalign

#endif
