// BF16 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   C[M, N] (+)= A[M, K] * B[N, K]^T        A, B: bf16, K contiguous
//
// One CTA of 128 threads owns a 128 x BN tile of C (BN = 16..128, multiple of
// 16).  K advances in chunks of 64 through a 3-stage ring: all threads copy
// the A and B chunks into shared memory with asynchronous 16-byte copies
// (cp.async, two chunks ahead of the one being multiplied) in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices; 128 B between core
// matrices along K, 1024 B between 8-row groups), one elected thread issues
// four tcgen05.mma (K = 16 each) into an FP32 accumulator in tensor memory and
// commits them to the stage's mbarrier, which frees the stage for the chunk
// three ahead.  The epilogue
// reads the accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 =
// rows of the tile), adds the bias, applies ReLU and stores FP32 or BF16.
// grid.z splits K (split-K partials go to C + z * split_stride).
//
// Every wait is bounded: a wait that gives up records kGemmTimeout in
// *status, the kernel still drains, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pdflow_gemm_tc.cuh"

namespace pdflow {
namespace {

constexpr int kBM = 128, kBK = 64, kMaxBN = 128, kThreads = 128;
constexpr uint32_t kTmemCols = 128;
constexpr int kStageA = kBM * kBK * 2;         // 16 KB
constexpr int kStageB = kMaxBN * kBK * 2;      // 16 KB at the widest N tile
constexpr int kStages = 3;
constexpr int kSmemBytes = kStages * (kStageA + kStageB) + 64;   // the attribute: the largest launch
// A launch's B stages hold only its N tile (bn rows), so narrow GEMMs fit
// more CTAs per SM (bn = 16: 55 KB, four CTAs, 4 x 128 TMEM columns = 512).
constexpr int smem_bytes(int bn) { return kStages * (kStageA + bn * kBK * 2) + 64; }
constexpr uint32_t kWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05 format): start address, leading
// byte offset (K direction), stride byte offset (M/N direction), all >> 4;
// bits 46-48 = 0b001; no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= uint64_t((addr >> 4) & 0x3FFFu);
    d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
    d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
    d |= uint64_t(1) << 46;
    return d;
}

// Instruction descriptor of kind::f16: D = F32, A = B = BF16, both K-major.
__device__ __forceinline__ uint32_t instr_desc(int bn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(bn >> 3) << 17) | (uint32_t(kBM >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity)
{
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Starts the asynchronous copy of rows [row0, row0 + rows) x K chunk
// [k0, k0 + 64) of a K-major bf16 matrix into the core-matrix layout; rows >=
// nrows and k >= K are zero-filled (source size 0, the source address is then
// the matrix base and nothing is read).  K is a multiple of 8, so a 16-byte
// piece is wholly inside or wholly outside.
__device__ __forceinline__ void stage_tile(unsigned char* dst, const __nv_bfloat16* src, int ld, int row0,
                                           int rows, int nrows, int k0, int K)
{
    const int chunks = rows * 8;   // 16-byte pieces
    for (int c = threadIdx.x; c < chunks; c += kThreads) {
        const int r = c % rows, kc = c / rows;
        const int gr = row0 + r, gk = k0 + kc * 8;
        const bool in = gr < nrows && gk < K;
        const __nv_bfloat16* g = in ? src + (size_t)gr * ld + gk : src;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                         smem_u32(dst + ((r >> 3) * 8 + kc) * 128 + (r & 7) * 16)),
                     "l"(g), "r"(in ? 16 : 0)
                     : "memory");
    }
}

// The pixel of an A row gathered by ConvGather: each thread stages the same
// row of every A tile (kThreads == kBM), so its (b, y, x) is found once.
struct ConvRow {
    int b, y, x;
    bool valid;
};

__device__ __forceinline__ ConvRow conv_row(const ConvGather& cv, int gr, int nrows)
{
    ConvRow cr;
    const int hw = cv.H * cv.W;
    cr.valid = gr < nrows;
    cr.b = gr / hw;
    const int rr = gr - cr.b * hw;
    cr.y = rr / cv.W;
    cr.x = rr - cr.y * cv.W;
    return cr;
}

// stage_tile for an A operand that is the im2col of a 3x3 convolution
// (ConvGather): each 16-byte piece is 8 channels of one tap of this thread's
// pixel, read from the NHWC source, or zero-filled outside the image, past
// row nrows or past K, exactly the values the materialised im2col holds.
__device__ __forceinline__ void stage_conv_tile(unsigned char* dst, const ConvGather& cv, const ConvRow& cr, int k0,
                                                int K)
{
    static_assert(kThreads == kBM, "one A row per thread");
    const __nv_bfloat16* s1 = static_cast<const __nv_bfloat16*>(cv.s1);
    const __nv_bfloat16* s2 = static_cast<const __nv_bfloat16*>(cv.s2);
    const int cin = cv.c1 + cv.c2;
    const int HH = cv.up1 ? cv.H1 : cv.H, WW = cv.up1 ? cv.W1 : cv.W;
    const int r = threadIdx.x;
    int tap = k0 / cin, ch = k0 - tap * cin;   // of piece 0; pieces step 8 channels
#pragma unroll
    for (int kc = 0; kc < kBK / 8; ++kc) {
        const int gk = k0 + kc * 8;
        const __nv_bfloat16* g = s1;   // read nothing (source size 0)
        bool in = cr.valid && gk < K;
        if (in) {
            const int h = cr.y + tap / 3 - 1, w = cr.x + tap % 3 - 1;
            in = h >= 0 && h < cv.H && w >= 0 && w < cv.W;
            if (in) {
                if (ch < cv.c1) {
                    const int hh = cv.up1 ? h / 2 : h, ww = cv.up1 ? w / 2 : w;
                    g = s1 + (((size_t)cr.b * HH + hh) * WW + ww) * cv.c1 + ch;
                } else {
                    g = s2 + (((size_t)cr.b * cv.H + h) * cv.W + w) * cv.c2 + (ch - cv.c1);
                }
            }
        }
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                         smem_u32(dst + ((r >> 3) * 8 + kc) * 128 + (r & 7) * 16)),
                     "l"(g), "r"(in ? 16 : 0)
                     : "memory");
        ch += 8;
        if (ch >= cin) {
            ch -= cin;
            ++tap;
        }
    }
}

__global__ void __launch_bounds__(kThreads, 1) k_gemm_tc(GemmArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    // stage i: A at smem + i * kStageA, B after all A stages
    auto sA = [&](int i) { return smem + i * kStageA; };
    const int stage_b = a.bn * kBK * 2;
    auto sB = [&](int i) { return smem + kStages * kStageA + i * stage_b; };
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kStages * (kStageA + stage_b));
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + kStages);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * a.bn;
    const int kbeg = blockIdx.z * a.k_per_split;
    const int kend = min(a.K, kbeg + a.k_per_split);
    const int nk = kend > kbeg ? (kend - kbeg + kBK - 1) / kBK : 0;

    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < kStages; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[i])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = instr_desc(a.bn);
    bool ok = true;

    const __nv_bfloat16* A = static_cast<const __nv_bfloat16*>(a.A);
    const ConvRow crow = a.conv_a ? conv_row(a.conv, m0 + (int)threadIdx.x, a.M) : ConvRow{0, 0, 0, false};
    const __nv_bfloat16* B = static_cast<const __nv_bfloat16*>(a.B);
    // prologue: chunks 0 .. kStages-2, one commit group each (empty past the end)
#pragma unroll
    for (int i = 0; i < kStages - 1; ++i) {
        if (i < nk) {
            if (a.conv_a) stage_conv_tile(sA(i), a.conv, crow, kbeg + i * kBK, kend);
            else stage_tile(sA(i), A, a.lda, m0, kBM, a.M, kbeg + i * kBK, kend);
            stage_tile(sB(i), B, a.ldb, n0, a.bn, a.N, kbeg + i * kBK, kend);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kStages;
        // groups committed so far: kStages - 1 + kc; chunk kc's is complete when
        // at most kStages - 2 younger ones are pending
        asm volatile("cp.async.wait_group %0;" ::"n"(kStages - 2) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            fence_after();
            const uint32_t abase = smem_u32(sA(s)), bbase = smem_u32(sB(s));
#pragma unroll
            for (int ks = 0; ks < kBK / 16; ++ks) {
                const uint64_t ad = smem_desc(abase + ks * 256, 128, 1024);
                const uint64_t bd = smem_desc(bbase + ks * 256, 128, 1024);
                const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[s]))
                         : "memory");
        }
        // refill: chunk kc + kStages - 1 goes into the stage chunk kc - 1 used,
        // once that chunk's multiplies have completed
        const int nc = kc + kStages - 1;
        if (nc < nk) {
            const int ns = nc % kStages;
            if (kc >= 1) ok &= mbar_wait(smem_u32(&mbar[ns]), uint32_t(((kc - 1) / kStages) & 1));
            if (a.conv_a) stage_conv_tile(sA(ns), a.conv, crow, kbeg + nc * kBK, kend);
            else stage_tile(sA(ns), A, a.lda, m0, kBM, a.M, kbeg + nc * kBK, kend);
            stage_tile(sB(ns), B, a.ldb, n0, a.bn, a.N, kbeg + nc * kBK, kend);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (nk > 0) ok &= mbar_wait(smem_u32(&mbar[(nk - 1) % kStages]), uint32_t(((nk - 1) / kStages) & 1));
    fence_after();

    // ---- epilogue: warp w holds rows 32w..32w+31 of the tile ----
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < a.bn; c0 += 16) {
        uint32_t r[16];
        const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < a.M && nk > 0) {
            const int col0 = n0 + c0;
            float v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float x = __uint_as_float(r[j]);
                if (a.bias && col0 + j < a.N) x += a.bias[col0 + j];
                if (a.relu) x = fmaxf(x, 0.f);
                v[j] = x;
            }
            if (a.out_bf16) {
                __nv_bfloat16* C = static_cast<__nv_bfloat16*>(a.C) + (size_t)row * a.ldc + col0;
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (col0 + j < a.N) C[j] = __float2bfloat16_rn(v[j]);
            } else {
                float* C =
                    static_cast<float*>(a.C) + (size_t)blockIdx.z * a.split_stride + (size_t)row * a.ldc + col0;
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (col0 + j < a.N) C[j] = v[j];
            }
        }
        __syncwarp();
    }
    if (!ok && lane == 0 && a.status) atomicExch(a.status, kGemmTimeout);

    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
    }
}

// Sums split-K partials [splits][M][ldc] into out [M][ldc] (fixed order).
__global__ void k_splitk_sum(const float* __restrict__ part, int splits, size_t stride, int M, int N, int ldc,
                             float* __restrict__ out)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)M * N) return;
    const size_t r = i / N, c = i % N, o = r * ldc + c;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[z * stride + o];
    out[o] = s;
}

}  // namespace

cudaError_t prepare_gemm_tc()
{
    return cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
}

cudaError_t launch_gemm_tc(const GemmArgs& args, cudaStream_t st)
{
    GemmArgs a = args;
    if (a.bn < 16 || a.bn > kMaxBN || (a.bn & 15) || (a.K & 7) || (a.lda & 7) || (a.ldb & 7) || a.M <= 0 ||
        a.N <= 0 || a.K <= 0)
        return cudaErrorInvalidValue;
    if (a.k_per_split <= 0) a.k_per_split = a.K;
    a.k_per_split = (a.k_per_split + kBK - 1) / kBK * kBK;
    const unsigned splits = (unsigned)((a.K + a.k_per_split - 1) / a.k_per_split);
    if (splits > 1 && a.out_bf16) return cudaErrorInvalidValue;
    dim3 grid((a.M + kBM - 1) / kBM, (a.N + a.bn - 1) / a.bn, splits);
    k_gemm_tc<<<grid, kThreads, smem_bytes(a.bn), st>>>(a);
    return cudaGetLastError();
}

unsigned gemm_splits(int K, int k_per_split)
{
    const int kp = (k_per_split + kBK - 1) / kBK * kBK;
    return (unsigned)((K + kp - 1) / kp);
}

cudaError_t launch_splitk_sum(const float* part, int splits, size_t stride, int M, int N, int ldc, float* out,
                              cudaStream_t st)
{
    const size_t n = (size_t)M * N;
    k_splitk_sum<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, splits, stride, M, N, ldc, out);
    return cudaGetLastError();
}

}  // namespace pdflow
