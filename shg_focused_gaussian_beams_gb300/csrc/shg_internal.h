// Internal declarations shared by the CUDA translation units and the host library.
#pragma once

#include <cuda_runtime.h>

#include <string>

namespace shg {

struct InstDesc;

constexpr int kMaxLine = 256;

// shg_march.cu
const float2 *twiddle_symbol_address();
cudaError_t launch_setup(const InstDesc *inst, int n_inst, int max_nn, int max_nz, cudaStream_t st);
cudaError_t launch_rows(int n, const InstDesc *inst, const int *list, int count, int s, cudaStream_t st);
cudaError_t launch_cols(int n, const InstDesc *inst, const int *list, int count, cudaStream_t st);
bool line_length_supported(int n);
cudaError_t launch_dft2d(int n, int sign, const float2 *in, float2 *out, cudaStream_t st);

// shg_host.cpp
void set_error(const std::string &msg);

}  // namespace shg
