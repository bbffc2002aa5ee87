/*
 * phpc_utils.h - host utilities of the drop-in (reference src/utils.h:6-7)
 * plus the seeded input generators and the closed-form known answer used by
 * the driver.
 */
#ifndef PHPC_UTILS_H
#define PHPC_UTILS_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference src/utils.c:9-17: current time in seconds (here a monotonic clock). */
double get_cur_time(void);

/* Reference src/utils.c:19-30: appends the 9-column row
 * N,size,gpu_count,num_blocks,threads_per_block,total_threads,cuda_time,cuda_gpu_time,cublas_time
 * with total_threads = gpu_count * num_blocks * threads_per_block. */
void log_to_csv(FILE *csv_file, int N, int size, int gpu_count, int num_blocks, int threads_per_block,
                double cuda_time, float cuda_gpu_time, double cublas_time);

/* Counter-based generator: element i of stream `seed` depends only on (seed, i),
 * so host and device (phpc_fill_*_dev in phpc_gemm.h) produce identical bits. */
uint64_t phpc_mix64(uint64_t x);
/* x[i] = uniform in [-1, 1) with 53 random bits, i = offset .. offset + n - 1. */
void phpc_fill_uniform(double *x, size_t n, uint64_t seed, uint64_t offset);
/* x[i] = u * 2^e, u uniform in [-1, 1), e uniform integer in [emin, emax]. */
void phpc_fill_wide(double *x, size_t n, uint64_t seed, uint64_t offset, int emin, int emax);
/* x[i] = i (the reference's inputs, src/main.c:85-86). */
void phpc_fill_index(double *x, size_t n);

/* Reference src/iterative.c:8-13: C += A * B for n x n row-major matrices on
 * the host, one thread, in the reference's loop order (the CPU timing of
 * bin/iterative.out). */
void phpc_gemm_iterative(const double *A, const double *B, double *C, int n);

/* Exact (A * B)[i][j] for A = B = index matrix of order n, rounded once to double:
 * i*n^2*S1 + i*j*n^2 + n*S2 + j*S1, S1 = n(n-1)/2, S2 = (n-1)n(2n-1)/6. */
double phpc_kat_index_entry(int n, int i, int j);

#ifdef __cplusplus
}
#endif

#endif /* PHPC_UTILS_H */
