// tcgen05 BF16 GEMM (pdflow_gemm_tc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace pdflow {

constexpr unsigned kGemmTimeout = 0x47454D4Du;   // status word written when a bounded wait gives up

// C[M, N] = A[M, K] * B[N, K]^T (+ bias[N], ReLU); A, B bf16 with K contiguous
// (lda, ldb and K multiples of 8); C fp32 or bf16 with leading dimension ldc.
// k_per_split < K splits K over grid.z (fp32 output only): split z writes its
// partial to C + z * split_stride.
// The A operand gathered while staging, as the im2col of a 3x3 "same"
// convolution, instead of read from a materialised [M][K] matrix: row p =
// pixel (b, y, x) of an n x H x W batch, column k = tap * (c1 + c2) + channel
// over [src1 (nearest-upsampled from H1 x W1 when up1) | src2], NHWC bf16 with
// channel counts multiples of 8 (16-byte pieces never straddle a tap).
struct ConvGather {
    const void* s1 = nullptr;
    const void* s2 = nullptr;
    int c1 = 0, c2 = 0, up1 = 0, H1 = 0, W1 = 0, H = 0, W = 0;
};

struct GemmArgs {
    const void* A = nullptr;
    const void* B = nullptr;
    int M = 0, N = 0, K = 0;
    int lda = 0, ldb = 0;
    void* C = nullptr;
    int ldc = 0;
    int out_bf16 = 0;
    const float* bias = nullptr;
    int relu = 0;
    int bn = 128;                 // N tile: 16..128, multiple of 16
    int k_per_split = 0;          // 0: no split
    size_t split_stride = 0;      // elements
    unsigned* status = nullptr;   // device word, kGemmTimeout on a bounded-wait timeout
    int conv_a = 0;               // 1: A is conv's im2col (A, lda unused)
    ConvGather conv;
};

cudaError_t prepare_gemm_tc();
cudaError_t launch_gemm_tc(const GemmArgs& a, cudaStream_t st);
unsigned gemm_splits(int K, int k_per_split);
cudaError_t launch_splitk_sum(const float* part, int splits, size_t stride, int M, int N, int ldc, float* out,
                              cudaStream_t st);

}  // namespace pdflow
