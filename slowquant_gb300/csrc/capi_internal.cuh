// capi_internal.cuh -- error-state helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include "../../include/slowquant_gb300.h"

namespace sq {

// Record a message for sq_last_error() (thread-local) and return `code`.
int set_error(int code, const char *fmt, ...);

// SQ_OK if the last launch succeeded, else SQ_ERR_CUDA with the CUDA message.
int check_launch(const char *what);

// y[i] = (float)x[i] on `stream`.
int to_float(long long n, const double *x, float *y, cudaStream_t stream);
int to_df(long long n, const double *x, float *y, cudaStream_t stream);

// sq_jk with every class launch on the caller's stream (no library stream pool).
int jk_serial(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
              const double *table64, const float *table32, const double *D, float *D32, double *Jacc, double *Kacc,
              int precision, void *stream);

}  // namespace sq
