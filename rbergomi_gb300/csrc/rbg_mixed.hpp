// rbg_mixed.hpp -- the mixed-precision form: tcgen05 Toeplitz-GEMM path
// kernel fused with Philox generation and the variance-path epilogue.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "rbg_internal.hpp"

namespace rbg {

struct MixedJob {
    int64_t batch = 0;           // paths per launch
    size_t workspace_bytes = 0;  // device workspace for tables and the error word
    int N = 0, n_vol = 0, n_vg = 0, split = 0;
    std::vector<unsigned char> host_ws;  // image uploaded by mixed_upload
    size_t off_err = 0;
};

int mixed_prepare(const Plan& plan, const rbg_options& o, int64_t M, MixedJob& job, std::string& err);
int mixed_upload(MixedJob& job, void* ws, cudaStream_t st, std::string& err);
int mixed_launch(const MixedJob& job, void* ws, uint64_t seed, int64_t path0, int64_t B, double* ivb,
                 cudaStream_t st, std::string& err);
int mixed_check(const MixedJob& job, void* ws, cudaStream_t st, std::string& err);
void mixed_release_cache();

}  // namespace rbg
