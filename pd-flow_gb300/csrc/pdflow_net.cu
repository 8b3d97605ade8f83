// Learned warm start: a 4-level convolutional encoder-decoder that predicts
// the 60x80 level's flow (du, dv in that level's pixels, dw in metres) from
// both frames' intensity and depth at that level, trained and run with this
// file's kernels.  Every convolution is an im2col + tcgen05 BF16 GEMM
// (pdflow_gemm_tc.cu) with FP32 accumulation; weights and activations are
// stored in BF16, FP32 master weights are updated by Adam.
//
// Image layout: the solver's column-major level planes (idx = v + u * 60)
// read as an 80 x 60 row-major image (h = u, w = v); activations are NHWC
// [n][h][w][c] with channel counts padded to multiples of 8.
//
//   enc1: 8(4 used) -> 16 -> 16      80x60   (skip1)
//   enc2: 16 -> 32 -> 32             40x30   (skip2)   2x2 average pooling between levels
//   enc3: 32 -> 64 -> 64             20x15   (skip3)   (ceil mode at odd sizes)
//   enc4: 64 -> 96 -> 96             10x8
//   dec3: [up(enc4) 96 | skip3 64] -> 64     20x15     nearest upsampling, cropped
//   dec2: [up(dec3) 64 | skip2 32] -> 32     40x30
//   dec1: [up(dec2) 32 | skip1 16] -> 16     80x60
//   head: 16 -> 3 (padded to 16), no ReLU, FP32 output
// 3x3 convolutions with zero padding; 338 k parameters.
#include <atomic>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/pdflow_net.h"
#include "pdflow_gemm_tc.cuh"
#include "pdflow_internal.h"
#include "pdflow_net.cuh"

using namespace pdflow;

namespace pdflow {
namespace {

constexpr int kH = 80, kW = 60, kHW = kH * kW;
constexpr float kWScale = 20.f;   // dw is learned as 20 * dw (metres) so all outputs are O(1)

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Solver-layout inputs [n][4][HW] (I1, I2 in 0..255, Z1, Z2 in metres) ->
// normalised bf16 NHWC [n][HW][8].
__global__ void k_net_input(const float* __restrict__ in, int n, __nv_bfloat16* __restrict__ x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kHW) return;
    const int b = i / kHW, p = i % kHW;
    const float* src = in + (size_t)b * 4 * kHW;
    __nv_bfloat16 v[8];
    v[0] = __float2bfloat16_rn(src[p] * (1.f / 255.f) - 0.5f);
    v[1] = __float2bfloat16_rn(src[kHW + p] * (1.f / 255.f) - 0.5f);
    const float z1 = src[2 * kHW + p], z2 = src[3 * kHW + p];
    v[2] = __float2bfloat16_rn(z1 > 0.f ? 0.5f * (z1 - 2.5f) : -1.5f);
    v[3] = __float2bfloat16_rn(z2 > 0.f ? 0.5f * (z2 - 2.5f) : -1.5f);
    for (int c = 4; c < 8; ++c) v[c] = __float2bfloat16_rn(0.f);
    *reinterpret_cast<uint4*>(x + (size_t)i * 8) = *reinterpret_cast<const uint4*>(v);
}

// The solver's pyramid planes at the 60x80 level -> net input [n][4][HW].
__global__ void k_gather_input(PyrLevel o, PyrLevel nw, size_t pstride, const unsigned* __restrict__ map, int n,
                               float* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kHW) return;
    const int b = i / kHW, p = i % kHW;
    const size_t po = pair_off(map, pstride, (unsigned)b);
    float* d = out + (size_t)b * 4 * kHW;
    d[p] = at(o.col, po)[p];
    d[kHW + p] = at(nw.col, po)[p];
    d[2 * kHW + p] = at(o.dep, po)[p];
    d[3 * kHW + p] = at(nw.dep, po)[p];
}

// im2col of a 3x3 "same" convolution over [src1 (optionally nearest-upsampled
// from H1 x W1) | src2]: col[p][tap * Cin + c], 16-byte chunks.
__global__ void k_im2col(const __nv_bfloat16* __restrict__ s1, int c1, int up1, int H1, int W1,
                         const __nv_bfloat16* __restrict__ s2, int c2, int n, int H, int W,
                         __nv_bfloat16* __restrict__ col)
{
    const int cin = c1 + c2, chunks = cin / 8;
    const size_t total = (size_t)n * H * W * 9 * chunks;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int ch = (int)(i % chunks);
    const int tap = (int)((i / chunks) % 9);
    const size_t p = i / ((size_t)chunks * 9);
    const int b = (int)(p / ((size_t)H * W)), r = (int)(p % ((size_t)H * W));
    const int h = r / W + tap / 3 - 1, w = r % W + tap % 3 - 1;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (h >= 0 && h < H && w >= 0 && w < W) {
        const int c = ch * 8;
        if (c < c1) {
            const int hh = up1 ? h / 2 : h, ww = up1 ? w / 2 : w;
            const int HH = up1 ? H1 : H, WW = up1 ? W1 : W;
            v = *reinterpret_cast<const uint4*>(s1 + (((size_t)b * HH + hh) * WW + ww) * c1 + c);
        } else {
            v = *reinterpret_cast<const uint4*>(s2 + (((size_t)b * H + h) * W + w) * c2 + (c - c1));
        }
    }
    *reinterpret_cast<uint4*>(col + p * (size_t)(9 * cin) + tap * cin + ch * 8) = v;
}

// Gradient of im2col: d_in[q][c] = sum over taps of dcol[q - off(tap)][tap * Cin + c]
// (FP32), written (not accumulated) into dcat [P][Cin].
__global__ void k_col2im(const float* __restrict__ dcol, int cin, int n, int H, int W, float* __restrict__ dcat)
{
    const size_t total = (size_t)n * H * W * cin;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c = (int)(i % cin);
    const size_t q = i / cin;
    const int b = (int)(q / ((size_t)H * W)), r = (int)(q % ((size_t)H * W));
    const int h = r / W, w = r % W;
    float s = 0.f;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int ph = h - (tap / 3 - 1), pw = w - (tap % 3 - 1);
        if (ph < 0 || ph >= H || pw < 0 || pw >= W) continue;
        const size_t p = ((size_t)b * H + ph) * W + pw;
        s += dcol[p * (size_t)(9 * cin) + tap * cin + c];
    }
    dcat[i] = s;
}

// Splits the concatenated input gradient: channels [c1, c1 + c2) are added to
// d2 (same resolution), channels [0, c1) to d1, summed over the 2x2 children
// when src1 was upsampled from H1 x W1.
__global__ void k_split_grad(const float* __restrict__ dcat, int c1, int c2, int up1, int H1, int W1, int n, int H,
                             int W, float* __restrict__ d1, float* __restrict__ d2)
{
    const int cin = c1 + c2;
    const size_t tot2 = (size_t)n * H * W * c2;
    const size_t tot1 = up1 ? (size_t)n * H1 * W1 * c1 : (size_t)n * H * W * c1;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < tot2 && d2) {
        const int c = (int)(i % c2);
        const size_t q = i / c2;
        d2[i] += dcat[q * cin + c1 + c];
    }
    if (i < tot1 && d1) {
        const int c = (int)(i % c1);
        const size_t q = i / c1;
        if (!up1) {
            d1[i] += dcat[q * cin + c];
        } else {
            const int b = (int)(q / ((size_t)H1 * W1)), r = (int)(q % ((size_t)H1 * W1));
            const int hh = r / W1, ww = r % W1;
            float s = 0.f;
            for (int dh = 0; dh < 2; ++dh)
                for (int dw = 0; dw < 2; ++dw) {
                    const int h = 2 * hh + dh, w = 2 * ww + dw;
                    if (h < H && w < W) s += dcat[(((size_t)b * H + h) * W + w) * cin + c];
                }
            d1[i] += s;
        }
    }
}

// 2x2 average pooling (ceil mode: the mean of the in-range taps), bf16.
__global__ void k_pool(const __nv_bfloat16* __restrict__ x, int C, int n, int H, int W, __nv_bfloat16* __restrict__ y)
{
    const int Ho = (H + 1) / 2, Wo = (W + 1) / 2;
    const size_t total = (size_t)n * Ho * Wo * C;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c = (int)(i % C);
    const size_t q = i / C;
    const int b = (int)(q / ((size_t)Ho * Wo)), r = (int)(q % ((size_t)Ho * Wo));
    const int ho = r / Wo, wo = r % Wo;
    float s = 0.f;
    int cnt = 0;
    for (int dh = 0; dh < 2; ++dh)
        for (int dw = 0; dw < 2; ++dw) {
            const int h = 2 * ho + dh, w = 2 * wo + dw;
            if (h < H && w < W) {
                s += __bfloat162float(x[(((size_t)b * H + h) * W + w) * C + c]);
                ++cnt;
            }
        }
    y[i] = __float2bfloat16_rn(s / (float)cnt);
}

// Gradient of k_pool, added into dx (FP32).
__global__ void k_pool_grad(const float* __restrict__ dy, int C, int n, int H, int W, float* __restrict__ dx)
{
    const size_t total = (size_t)n * H * W * C;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c = (int)(i % C);
    const size_t q = i / C;
    const int b = (int)(q / ((size_t)H * W)), r = (int)(q % ((size_t)H * W));
    const int h = r / W, w = r % W;
    const int Ho = (H + 1) / 2, Wo = (W + 1) / 2, ho = h / 2, wo = w / 2;
    const int cnt = (min(2 * ho + 2, H) - 2 * ho) * (min(2 * wo + 2, W) - 2 * wo);
    dx[i] += dy[(((size_t)b * Ho + ho) * Wo + wo) * C + c] / (float)cnt;
}

// dY (bf16) = dA * relu'(A) (A the layer's bf16 output); no mask for the head.
__global__ void k_relu_grad(const float* __restrict__ da, const __nv_bfloat16* __restrict__ a, size_t count,
                            __nv_bfloat16* __restrict__ dy)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float g = (!a || __bfloat162float(a[i]) > 0.f) ? da[i] : 0.f;
    dy[i] = __float2bfloat16_rn(g);
}

// out[c][r] = in[r][c] for a rows x cols bf16 matrix (32 x 32 tiles); out's
// rows are rows_pad long, zero beyond `rows`.
__global__ void k_transpose(const __nv_bfloat16* __restrict__ in, size_t rows, size_t rows_pad, int cols,
                            __nv_bfloat16* __restrict__ out)
{
    __shared__ __nv_bfloat16 t[32][33];
    const size_t r0 = (size_t)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const size_t r = r0 + k;
        const int c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[k][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k;
        const size_t r = r0 + threadIdx.x;
        if (r < rows_pad && c < cols)
            out[(size_t)c * rows_pad + r] = r < rows ? t[threadIdx.x][k] : __float2bfloat16_rn(0.f);
    }
}

// Column sums of dY [P][C] (bias gradients); one block per channel, fixed order.
__global__ void k_colsum(const __nv_bfloat16* __restrict__ dy, size_t P, int C, float* __restrict__ out)
{
    const int c = blockIdx.x;
    float s = 0.f;
    for (size_t p = threadIdx.x; p < P; p += blockDim.x) s += __bfloat162float(dy[p * C + c]);
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}

// Masked mean-squared error of the head output [P][16] against labels
// [n][3][HW] (du, dv, 20 dw) on pixels whose old depth is valid; writes
// dOut and one partial loss per block.
__global__ void k_loss(const float* __restrict__ out, const float* __restrict__ label, const float* __restrict__ input,
                       int n, float inv_count, float* __restrict__ dout, float* __restrict__ partial)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n * kHW) {
        const int b = i / kHW, p = i % kHW;
        const bool valid = input[(size_t)b * 4 * kHW + 2 * kHW + p] > 0.f;
        for (int c = 0; c < 16; ++c) {
            float g = 0.f;
            if (c < 3 && valid) {
                const float t = label[(size_t)b * 3 * kHW + c * kHW + p] * (c == 2 ? kWScale : 1.f);
                const float d = out[(size_t)i * 16 + c] - t;
                l += d * d;
                g = 2.f * d * inv_count;
            }
            dout[(size_t)i * 16 + c] = g;
        }
    }
    __shared__ float red[256];
    red[threadIdx.x] = l;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_valid_count(const float* __restrict__ input, int n, unsigned* __restrict__ count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kHW) return;
    const int b = i / kHW, p = i % kHW;
    if (input[(size_t)b * 4 * kHW + 2 * kHW + p] > 0.f) atomicAdd(count, 1u);
}

// Head output [P][16] -> solver seed / user output [n][3][HW] (du, dv, dw).
__global__ void k_head_out(const float* __restrict__ out, int n, float* __restrict__ seed)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kHW) return;
    const int b = i / kHW, p = i % kHW;
    float* s = seed + (size_t)b * 3 * kHW;
    s[p] = out[(size_t)i * 16];
    s[kHW + p] = out[(size_t)i * 16 + 1];
    s[2 * kHW + p] = out[(size_t)i * 16 + 2] * (1.f / kWScale);
}

// Adam on FP32 master weights w [cout][k] (gradient in the GEMM's transposed
// layout gT [k][cout_pad]), then the bf16 copies W [cout_pad][k] and
// WT [k][cout_pad] (padding rows stay zero).
__global__ void k_adam_w(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                         const float* __restrict__ gT, int cout, int cout_pad, int k, float lr, float b1, float b2,
                         float eps, float c1, float c2, int update, __nv_bfloat16* __restrict__ W,
                         __nv_bfloat16* __restrict__ WT)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cout * k) return;
    const int o = i / k, j = i % k;
    float x = w[i];
    if (update) {
        const float g = gT[(size_t)j * cout_pad + o];
        const float mm = b1 * m[i] + (1.f - b1) * g;
        const float vv = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mm;
        v[i] = vv;
        x -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        w[i] = x;
    }
    const __nv_bfloat16 q = __float2bfloat16_rn(x);
    W[(size_t)o * k + j] = q;
    WT[(size_t)j * cout_pad + o] = q;
}

__global__ void k_adam_b(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                         const float* __restrict__ g, int count, float lr, float b1, float b2, float eps, float c1,
                         float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gg = g[i];
    const float mm = b1 * m[i] + (1.f - b1) * gg;
    const float vv = b2 * v[i] + (1.f - b2) * gg * gg;
    m[i] = mm;
    v[i] = vv;
    w[i] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// Head bias: added to the FP32 head output in place (3 real channels).
__global__ void k_head_bias(float* head, size_t P, const float* bias)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P * 3) return;
    head[(i / 3) * 16 + i % 3] += bias[i % 3];
}

unsigned blocks(size_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace
}  // namespace pdflow

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

struct Conv {
    // input: [src1 (c1, upsampled from the coarser level if up1) | src2 (c2)]
    int src1, c1, up1, src2, c2;     // activation ids (-1: none)
    int cout, cout_pad;              // real / padded output channels
    int H, W;                        // output (= input) resolution
    int relu;
    int out;                         // activation id written
    int K() const { return 9 * (c1 + c2); }
    size_t woff = 0, boff = 0;       // offsets of weights [cout][K] and bias [cout] in the parameter vector
};

struct Act {
    int C, H, W;
    __nv_bfloat16* x = nullptr;      // [n][H][W][C]
    float* g = nullptr;              // gradient [n][H][W][C]
};

}  // namespace

struct pdflow_net {
    unsigned long long uid = 0;      // unique per created network (key of graphs that read it)
    unsigned max_batch = 0;
    cudaStream_t stream = nullptr;
    std::vector<Act> act;
    std::vector<Conv> conv;
    struct Pool { int in, out; };
    std::vector<Pool> pools;
    size_t nparams = 0;
    // device buffers
    float *w = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;   // fp32 [nparams]
    std::vector<__nv_bfloat16*> Wb, WTb;                               // per conv bf16 weights
    std::vector<float*> gT;                                            // per conv dW^T [K][cout_pad]
    __nv_bfloat16 *col = nullptr, *colT = nullptr, *dy = nullptr, *dyT = nullptr;
    float *dcol = nullptr, *dcat = nullptr, *head = nullptr, *dhead = nullptr, *part = nullptr;
    float *loss_part = nullptr, *input = nullptr;
    unsigned* count = nullptr;
    unsigned* status = nullptr;
    size_t col_elems = 0, part_elems = 0;
    int step = 0;
    size_t device_bytes = 0;
    std::vector<void*> allocs;
};

namespace {

thread_local std::string g_net_error;

// The GEMM kernel's shared-memory attribute, once per device, under a lock.
cudaError_t prepare_gemm_once()
{
    static std::mutex mu;
    static unsigned long long prepared = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && ((prepared >> dev) & 1ull)) return cudaSuccess;
    e = prepare_gemm_tc();
    if (e == cudaSuccess && dev < 64) prepared |= 1ull << dev;
    return e;
}

int net_fail(int code, const char* what, cudaError_t e = cudaSuccess)
{
    g_net_error = what;
    if (e != cudaSuccess) {
        g_net_error += ": ";
        g_net_error += cudaGetErrorString(e);
    }
    pdflow::set_last_error(g_net_error.c_str());
    return code;
}

#define NET_TRY(call, what)                                                      \
    do {                                                                         \
        cudaError_t _e = (call);                                                 \
        if (_e != cudaSuccess) return net_fail(PDFLOW_ERR_CUDA, what, _e);        \
    } while (0)

int add_act(pdflow_net* n, int C, int H, int W)
{
    n->act.push_back(Act{C, H, W});
    return int(n->act.size()) - 1;
}

void build_graph(pdflow_net* n)
{
    const int H0 = kH, W0 = kW, H1 = 40, W1 = 30, H2 = 20, W2 = 15, H3 = 10, W3 = 8;
    const int x0 = add_act(n, 8, H0, W0);
    auto conv = [&](int s1, int up1, int s2, int cout, int cout_pad, int H, int W, int relu) {
        Conv c{};
        c.src1 = s1;
        c.c1 = n->act[s1].C;
        c.up1 = up1;
        c.src2 = s2;
        c.c2 = s2 >= 0 ? n->act[s2].C : 0;
        c.cout = cout;
        c.cout_pad = cout_pad;
        c.H = H;
        c.W = W;
        c.relu = relu;
        c.out = add_act(n, cout_pad, H, W);
        n->conv.push_back(c);
        return c.out;
    };
    auto pool = [&](int in, int H, int W) {
        const int o = add_act(n, n->act[in].C, H, W);
        n->pools.push_back({in, o});
        return o;
    };
    const int e1a = conv(x0, 0, -1, 16, 16, H0, W0, 1);
    const int e1b = conv(e1a, 0, -1, 16, 16, H0, W0, 1);
    const int p1 = pool(e1b, H1, W1);
    const int e2a = conv(p1, 0, -1, 32, 32, H1, W1, 1);
    const int e2b = conv(e2a, 0, -1, 32, 32, H1, W1, 1);
    const int p2 = pool(e2b, H2, W2);
    const int e3a = conv(p2, 0, -1, 64, 64, H2, W2, 1);
    const int e3b = conv(e3a, 0, -1, 64, 64, H2, W2, 1);
    const int p3 = pool(e3b, H3, W3);
    const int e4a = conv(p3, 0, -1, 96, 96, H3, W3, 1);
    const int e4b = conv(e4a, 0, -1, 96, 96, H3, W3, 1);
    const int d3 = conv(e4b, 1, e3b, 64, 64, H2, W2, 1);
    const int d2 = conv(d3, 1, e2b, 32, 32, H1, W1, 1);
    const int d1 = conv(d2, 1, e1b, 16, 16, H0, W0, 1);
    conv(d1, 0, -1, 3, 16, H0, W0, 0);
    size_t off = 0;
    for (auto& c : n->conv) {
        c.woff = off;
        off += size_t(c.cout) * c.K();
        c.boff = off;
        off += c.cout;
    }
    n->nparams = off;
}

// splitmix64 + Box-Muller: He-normal initial weights from a seed.
void init_params(pdflow_net* n, unsigned long long seed, std::vector<float>& h)
{
    h.assign(n->nparams, 0.f);
    uint64_t s = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (auto& c : n->conv) {
        const int cin_used = (c.src1 == 0) ? 4 : c.c1 + c.c2;
        const double sd = std::sqrt(2.0 / (9.0 * cin_used)) * (c.relu ? 1.0 : 0.1);
        const int cin = c.c1 + c.c2;
        for (int o = 0; o < c.cout; ++o)
            for (int k = 0; k < c.K(); ++k) {
                const int ci = k % cin;
                double g = 0.0;
                if (!(c.src1 == 0 && ci >= 4)) {
                    const double u1 = next() + 1e-300, u2 = next();
                    g = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2) * sd;
                }
                h[c.woff + size_t(o) * c.K() + k] = float(g);
            }
    }
}

int upload_params(pdflow_net* n)
{
    cudaStream_t st = n->stream;
    for (size_t i = 0; i < n->conv.size(); ++i) {
        const Conv& c = n->conv[i];
        k_adam_w<<<blocks(size_t(c.cout) * c.K()), 256, 0, st>>>(n->w + c.woff, nullptr, nullptr, nullptr, c.cout,
                                                                  c.cout_pad, c.K(), 0.f, 0.f, 0.f, 0.f, 1.f, 1.f, 0,
                                                                  n->Wb[i], n->WTb[i]);
        NET_TRY(cudaGetLastError(), "weight conversion launch");
    }
    return PDFLOW_OK;
}

template <class T>
T* dalloc(pdflow_net* n, size_t count, cudaError_t* e)
{
    void* p = nullptr;
    if (*e == cudaSuccess) *e = cudaMalloc(&p, count * sizeof(T) + 16);
    if (*e == cudaSuccess) {
        n->allocs.push_back(p);
        n->device_bytes += count * sizeof(T) + 16;
        *e = cudaMemset(p, 0, count * sizeof(T) + 16);
    }
    return static_cast<T*>(p);
}

// From this many inputs on, a convolution's GEMM gathers its im2col operand
// while staging it (no im2col kernel, no column matrix round trip: 48.06 ->
// 47.73 ms per 64-pair learned VGA solve); below it the separate im2col kernel
// is faster (one pair: 2.035 against 2.083 ms), as the small GEMM is
// latency-bound.  Both give the same bits.
constexpr int kImplicitConvMinBatch = 16;

int conv_forward(pdflow_net* n, const Conv& c, size_t ci, int nb)
{
    cudaStream_t st = n->stream;
    const Act& o = n->act[c.out];
    const Act& a1 = n->act[c.src1];
    const Act* a2 = c.src2 >= 0 ? &n->act[c.src2] : nullptr;
    const size_t P = size_t(nb) * c.H * c.W;
    const int K = c.K();
    GemmArgs g;
    if (nb >= kImplicitConvMinBatch) {
        g.conv_a = 1;
        g.conv.s1 = a1.x;
        g.conv.s2 = a2 ? a2->x : nullptr;
        g.conv.c1 = c.c1;
        g.conv.c2 = c.c2;
        g.conv.up1 = c.up1;
        g.conv.H1 = a1.H;
        g.conv.W1 = a1.W;
        g.conv.H = c.H;
        g.conv.W = c.W;
        g.A = a1.x;
    } else {
        k_im2col<<<blocks(P * 9 * (K / 72)), 256, 0, st>>>(a1.x, c.c1, c.up1, a1.H, a1.W, a2 ? a2->x : nullptr,
                                                           c.c2, nb, c.H, c.W, n->col);
        NET_TRY(cudaGetLastError(), "im2col launch");
        g.A = n->col;
    }
    g.B = n->Wb[ci];
    g.M = int(P);
    g.N = c.cout_pad;
    g.K = K;
    g.lda = K;
    g.ldb = K;
    g.relu = c.relu;
    g.bn = c.cout_pad;
    g.status = n->status;
    if (c.cout == c.cout_pad) {          // hidden layer: bias + ReLU, bf16 activation
        g.bias = n->w + c.boff;
        g.C = o.x;
        g.ldc = c.cout_pad;
        g.out_bf16 = 1;
    } else {                             // head: FP32, bias added by k_head_bias
        g.C = n->head;
        g.ldc = 16;
    }
    NET_TRY(launch_gemm_tc(g, st), "conv GEMM launch");
    return PDFLOW_OK;
}

}  // namespace

namespace pdflow {

// Forward pass over nb inputs [nb][4][HW] (device); leaves the head output
// [nb*HW][16] (bias included) in n->head.
int net_forward(pdflow_net* n, int nb, const float* input)
{
    cudaStream_t st = n->stream;
    k_net_input<<<blocks(size_t(nb) * kHW), 256, 0, st>>>(input, nb, n->act[0].x);
    NET_TRY(cudaGetLastError(), "net input launch");
    size_t ci = 0;
    size_t pi = 0;
    // conv/pool order of build_graph: pools follow e1b, e2b, e3b
    const int pool_after[3] = {1, 3, 5};
    for (; ci < n->conv.size(); ++ci) {
        int rc = conv_forward(n, n->conv[ci], ci, nb);
        if (rc) return rc;
        if (pi < 3 && int(ci) == pool_after[pi]) {
            const auto& pl = n->pools[pi];
            const Act& a = n->act[pl.in];
            const Act& b = n->act[pl.out];
            k_pool<<<blocks(size_t(nb) * b.H * b.W * b.C), 256, 0, st>>>(a.x, a.C, nb, a.H, a.W, b.x);
            NET_TRY(cudaGetLastError(), "pool launch");
            ++pi;
        }
    }
    return PDFLOW_OK;
}

}  // namespace pdflow

namespace {

int forward_full(pdflow_net* n, int nb, const float* input)
{
    int rc = pdflow::net_forward(n, nb, input);
    if (rc) return rc;
    const Conv& h = n->conv.back();
    k_head_bias<<<blocks(size_t(nb) * kHW * 3), 256, 0, n->stream>>>(n->head, size_t(nb) * kHW, n->w + h.boff);
    NET_TRY(cudaGetLastError(), "head bias launch");
    return PDFLOW_OK;
}

// Backward pass from n->dhead ([P][16], FP32): fills n->gT (dW^T per conv)
// and n->grad bias entries.
int backward(pdflow_net* n, int nb)
{
    cudaStream_t st = n->stream;
    for (auto& a : n->act)
        if (a.g) NET_TRY(cudaMemsetAsync(a.g, 0, sizeof(float) * size_t(nb) * a.H * a.W * a.C, st), "grad reset");
    const int pool_after[3] = {1, 3, 5};
    for (int ci = int(n->conv.size()) - 1; ci >= 0; --ci) {
        const Conv& c = n->conv[ci];
        const size_t P = size_t(nb) * c.H * c.W;
        const int K = c.K();
        // pooling that consumed this layer's output: its gradient flows back first
        for (int q = 0; q < 3; ++q)
            if (pool_after[q] == ci) {
                const auto& pl = n->pools[q];
                const Act& a = n->act[pl.in];
                const Act& b = n->act[pl.out];
                k_pool_grad<<<blocks(size_t(nb) * a.H * a.W * a.C), 256, 0, st>>>(b.g, a.C, nb, a.H, a.W, a.g);
                NET_TRY(cudaGetLastError(), "pool grad launch");
            }
        // dY = dA * relu'(A)  (head: dY = dOut)
        const Act& o = n->act[c.out];
        if (c.relu)
            k_relu_grad<<<blocks(P * c.cout_pad), 256, 0, st>>>(o.g, o.x, P * c.cout_pad, n->dy);
        else
            k_relu_grad<<<blocks(P * 16), 256, 0, st>>>(n->dhead, nullptr, P * 16, n->dy);
        NET_TRY(cudaGetLastError(), "relu grad launch");
        // bias gradient
        k_colsum<<<c.cout, 256, 0, st>>>(n->dy, P, c.cout_pad, n->grad + c.boff);
        NET_TRY(cudaGetLastError(), "bias grad launch");
        // weight gradient: dW^T [K][cout_pad] = col^T [K][P] * dY^T [cout_pad][P]^T
        {
            const Act& a1 = n->act[c.src1];
            const Act* a2 = c.src2 >= 0 ? &n->act[c.src2] : nullptr;
            k_im2col<<<blocks(P * 9 * (K / 72)), 256, 0, st>>>(a1.x, c.c1, c.up1, a1.H, a1.W, a2 ? a2->x : nullptr,
                                                               c.c2, nb, c.H, c.W, n->col);
            NET_TRY(cudaGetLastError(), "im2col launch");
            // the transposed operands have P (the GEMM's K) padded to a multiple of 8 with zeros
            const size_t Pp = (P + 7) / 8 * 8;
            dim3 tb(32, 8);
            k_transpose<<<dim3(unsigned((Pp + 31) / 32), unsigned((K + 31) / 32)), tb, 0, st>>>(n->col, P, Pp, K,
                                                                                                n->colT);
            k_transpose<<<dim3(unsigned((Pp + 31) / 32), unsigned((c.cout_pad + 31) / 32)), tb, 0, st>>>(
                n->dy, P, Pp, c.cout_pad, n->dyT);
            NET_TRY(cudaGetLastError(), "transpose launch");
            GemmArgs g;
            g.A = n->colT;
            g.B = n->dyT;
            g.M = K;
            g.N = c.cout_pad;
            g.K = int(Pp);
            g.lda = int(Pp);
            g.ldb = int(Pp);
            g.C = n->part;
            g.ldc = c.cout_pad;
            g.bn = c.cout_pad;
            const int target_splits = 256 / ((K + 127) / 128);
            int kps = int((Pp + target_splits - 1) / target_splits);
            kps = (kps + 63) / 64 * 64;
            g.k_per_split = kps;
            g.split_stride = size_t(K) * c.cout_pad;
            g.status = n->status;
            const unsigned splits = gemm_splits(int(Pp), kps);
            if (size_t(splits) * g.split_stride > n->part_elems) return net_fail(PDFLOW_ERR_ARG, "split-K buffer");
            NET_TRY(launch_gemm_tc(g, st), "weight-gradient GEMM launch");
            NET_TRY(launch_splitk_sum(n->part, int(splits), g.split_stride, K, c.cout_pad, c.cout_pad, n->gT[ci], st),
                    "split-K sum launch");
        }
        if (ci == 0) break;   // no gradient w.r.t. the input
        // input gradient: dCol [P][K] = dY [P][cout_pad] * W^T  (B = WT [K][cout_pad])
        {
            GemmArgs g;
            g.A = n->dy;
            g.B = n->WTb[ci];
            g.M = int(P);
            g.N = K;
            g.K = c.cout_pad;
            g.lda = c.cout_pad;
            g.ldb = c.cout_pad;
            g.C = n->dcol;
            g.ldc = K;
            g.bn = 128;
            g.status = n->status;
            NET_TRY(launch_gemm_tc(g, st), "input-gradient GEMM launch");
            const int cin = c.c1 + c.c2;
            k_col2im<<<blocks(P * cin), 256, 0, st>>>(n->dcol, cin, nb, c.H, c.W, n->dcat);
            NET_TRY(cudaGetLastError(), "col2im launch");
            const Act& a1 = n->act[c.src1];
            const size_t t1 = c.up1 ? size_t(nb) * a1.H * a1.W * c.c1 : P * c.c1;
            const size_t t2 = P * c.c2;
            k_split_grad<<<blocks(t1 > t2 ? t1 : t2), 256, 0, st>>>(n->dcat, c.c1, c.c2, c.up1, a1.H, a1.W, nb, c.H,
                                                                     c.W, a1.g,
                                                                     c.src2 >= 0 ? n->act[c.src2].g : nullptr);
            NET_TRY(cudaGetLastError(), "split grad launch");
        }
    }
    return PDFLOW_OK;
}

int loss_and_grad(pdflow_net* n, int nb, const float* input, const float* label, float* loss_host)
{
    cudaStream_t st = n->stream;
    NET_TRY(cudaMemsetAsync(n->count, 0, sizeof(unsigned), st), "count reset");
    k_valid_count<<<blocks(size_t(nb) * kHW), 256, 0, st>>>(input, nb, n->count);
    unsigned cnt = 0;
    NET_TRY(cudaMemcpyAsync(&cnt, n->count, sizeof cnt, cudaMemcpyDeviceToHost, st), "count read");
    NET_TRY(cudaStreamSynchronize(st), "synchronize");
    const float inv = cnt ? 1.f / (3.f * float(cnt)) : 0.f;
    const unsigned nbk = blocks(size_t(nb) * kHW);
    k_loss<<<nbk, 256, 0, st>>>(n->head, label, input, nb, inv, n->dhead, n->loss_part);
    NET_TRY(cudaGetLastError(), "loss launch");
    if (loss_host) {
        std::vector<float> parts(nbk);
        NET_TRY(cudaMemcpyAsync(parts.data(), n->loss_part, sizeof(float) * nbk, cudaMemcpyDeviceToHost, st),
                "loss read");
        NET_TRY(cudaStreamSynchronize(st), "synchronize");
        double s = 0.0;
        for (float p : parts) s += p;
        *loss_host = float(s * inv);
    }
    return PDFLOW_OK;
}

int check_net_status(pdflow_net* n)
{
    unsigned s = 0;
    NET_TRY(cudaMemcpyAsync(&s, n->status, sizeof s, cudaMemcpyDeviceToHost, n->stream), "status read");
    NET_TRY(cudaStreamSynchronize(n->stream), "synchronize");
    if (s) {
        cudaMemsetAsync(n->status, 0, sizeof s, n->stream);
        cudaStreamSynchronize(n->stream);
        return net_fail(PDFLOW_ERR_TIMEOUT, "a tensor-core GEMM's bounded wait gave up");
    }
    return PDFLOW_OK;
}

}  // namespace

namespace pdflow {

int net_seed(pdflow_net* n, int nb, const float* input, float* seed)
{
    int rc = forward_full(n, nb, input);
    if (rc) return rc;
    k_head_out<<<blocks(size_t(nb) * kHW), 256, 0, n->stream>>>(n->head, nb, seed);
    NET_TRY(cudaGetLastError(), "head output launch");
    return PDFLOW_OK;
}

cudaError_t launch_gather_seed_input(const PyrLevel& o, const PyrLevel& nw, size_t pstride, const unsigned* map,
                                     int nb, float* out, cudaStream_t st)
{
    k_gather_input<<<blocks(size_t(nb) * kHW), 256, 0, st>>>(o, nw, pstride, map, nb, out);
    return cudaGetLastError();
}

int net_gather_input(pdflow_net* n, const PyrLevel& o, const PyrLevel& nw, size_t pstride, const unsigned* map,
                     int nb, cudaStream_t st)
{
    NET_TRY(launch_gather_seed_input(o, nw, pstride, map, nb, n->input, st), "net input gather launch");
    return PDFLOW_OK;
}

float* net_input_buffer(pdflow_net* n) { return n->input; }
unsigned net_max_batch(const pdflow_net* n) { return n->max_batch; }
unsigned long long net_uid(const pdflow_net* n) { return n->uid; }
unsigned net_seed_launches(const pdflow_net* n, int nb)
{
    // input, per convolution (im2col +) GEMM, pools, head bias, head output
    const unsigned convs = unsigned(n->conv.size());
    return 1u + convs * (nb >= kImplicitConvMinBatch ? 1u : 2u) + unsigned(n->pools.size()) + 2u;
}
cudaStream_t net_stream(const pdflow_net* n) { return n->stream; }
void net_set_stream_internal(pdflow_net* n, cudaStream_t st) { n->stream = st; }

}  // namespace pdflow

// ---------------------------------------------------------------------------
// C ABI (include/pdflow_net.h)
// ---------------------------------------------------------------------------
extern "C" {

int pdflow_net_create(unsigned max_batch, unsigned long long seed, pdflow_net** out)
{
    if (!out) return net_fail(PDFLOW_ERR_ARG, "null output handle");
    *out = nullptr;
    if (max_batch == 0 || max_batch > 4096) return net_fail(PDFLOW_ERR_ARG, "batch must be 1..4096");
    int dev = 0;
    NET_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop;
    NET_TRY(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    if (!(prop.major == 10 && prop.minor == 3))
        return net_fail(PDFLOW_ERR_NO_DEVICE, "this library is built for sm_103a (GB300) only");
    NET_TRY(prepare_gemm_once(), "GEMM kernel attributes");
    pdflow_net* n = new (std::nothrow) pdflow_net();
    static std::atomic<unsigned long long> next_uid{1};
    if (n) n->uid = next_uid++;
    if (!n) return net_fail(PDFLOW_ERR_OOM, "host allocation");
    n->max_batch = max_batch;
    build_graph(n);
    cudaError_t e = cudaSuccess;
    const size_t B = max_batch;
    n->w = dalloc<float>(n, n->nparams, &e);
    n->m = dalloc<float>(n, n->nparams, &e);
    n->v = dalloc<float>(n, n->nparams, &e);
    n->grad = dalloc<float>(n, n->nparams, &e);
    size_t maxK = 0, maxPK = 0, maxPcin = 0;
    for (auto& c : n->conv) {
        n->Wb.push_back(dalloc<__nv_bfloat16>(n, size_t(c.cout_pad) * c.K(), &e));
        n->WTb.push_back(dalloc<__nv_bfloat16>(n, size_t(c.K()) * c.cout_pad, &e));
        n->gT.push_back(dalloc<float>(n, size_t(c.K()) * c.cout_pad, &e));
        const size_t P = B * c.H * c.W, Pp = (P + 7) / 8 * 8;
        maxK = std::max(maxK, size_t(c.K()) * c.cout_pad);
        maxPK = std::max(maxPK, Pp * c.K());
        maxPcin = std::max(maxPcin, P * (c.c1 + c.c2));
    }
    for (auto& a : n->act) {
        a.x = dalloc<__nv_bfloat16>(n, B * a.H * a.W * a.C, &e);
        a.g = dalloc<float>(n, B * a.H * a.W * a.C, &e);
    }
    n->col_elems = maxPK;
    n->col = dalloc<__nv_bfloat16>(n, maxPK, &e);
    n->colT = dalloc<__nv_bfloat16>(n, maxPK, &e);
    n->dcol = dalloc<float>(n, maxPK, &e);
    n->dcat = dalloc<float>(n, maxPcin, &e);
    n->dy = dalloc<__nv_bfloat16>(n, B * kHW * 96, &e);
    n->dyT = dalloc<__nv_bfloat16>(n, B * kHW * 96, &e);
    n->head = dalloc<float>(n, B * kHW * 16, &e);
    n->dhead = dalloc<float>(n, B * kHW * 16, &e);
    n->part_elems = 300 * maxK;
    n->part = dalloc<float>(n, n->part_elems, &e);
    n->loss_part = dalloc<float>(n, B * kHW / 256 + 2, &e);
    n->input = dalloc<float>(n, B * 4 * kHW, &e);
    n->count = dalloc<unsigned>(n, 4, &e);
    n->status = dalloc<unsigned>(n, 4, &e);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        pdflow_net_destroy(n);
        return net_fail(PDFLOW_ERR_OOM, "device allocation", e);
    }
    std::vector<float> h;
    init_params(n, seed, h);
    int rc = pdflow_net_set_params(n, h.data(), h.size());
    if (rc) {
        pdflow_net_destroy(n);
        return rc;
    }
    *out = n;
    return PDFLOW_OK;
}

int pdflow_net_destroy(pdflow_net* n)
{
    if (!n) return PDFLOW_OK;
    if (n->stream) {
        cudaStreamSynchronize(n->stream);
        cudaStreamDestroy(n->stream);
    }
    for (void* p : n->allocs) cudaFree(p);
    delete n;
    return PDFLOW_OK;
}

size_t pdflow_net_param_count(const pdflow_net* n) { return n ? n->nparams : 0; }

size_t pdflow_net_device_bytes(const pdflow_net* n) { return n ? n->device_bytes : 0; }

int pdflow_net_set_params(pdflow_net* n, const float* params, size_t count)
{
    if (!n || !params) return net_fail(PDFLOW_ERR_ARG, "null argument");
    if (count != n->nparams) return net_fail(PDFLOW_ERR_ARG, "parameter count mismatch");
    NET_TRY(cudaMemcpyAsync(n->w, params, sizeof(float) * count, cudaMemcpyHostToDevice, n->stream), "H2D params");
    NET_TRY(cudaMemsetAsync(n->m, 0, sizeof(float) * count, n->stream), "adam reset");
    NET_TRY(cudaMemsetAsync(n->v, 0, sizeof(float) * count, n->stream), "adam reset");
    n->step = 0;
    int rc = upload_params(n);
    if (rc) return rc;
    NET_TRY(cudaStreamSynchronize(n->stream), "synchronize");
    return PDFLOW_OK;
}

int pdflow_net_get_params(pdflow_net* n, float* params, size_t count)
{
    if (!n || !params) return net_fail(PDFLOW_ERR_ARG, "null argument");
    if (count != n->nparams) return net_fail(PDFLOW_ERR_ARG, "parameter count mismatch");
    NET_TRY(cudaMemcpyAsync(params, n->w, sizeof(float) * count, cudaMemcpyDeviceToHost, n->stream), "D2H params");
    NET_TRY(cudaStreamSynchronize(n->stream), "synchronize");
    return PDFLOW_OK;
}

int pdflow_net_set_stream(pdflow_net* n, void* stream)
{
    if (!n) return net_fail(PDFLOW_ERR_ARG, "null handle");
    if (!stream) return net_fail(PDFLOW_ERR_ARG, "null stream");
    n->stream = static_cast<cudaStream_t>(stream);
    return PDFLOW_OK;
}

int pdflow_net_forward(pdflow_net* n, unsigned nb, const float* d_input, float* d_output)
{
    if (!n || !d_input || !d_output) return net_fail(PDFLOW_ERR_ARG, "null argument");
    if (nb == 0 || nb > n->max_batch) return net_fail(PDFLOW_ERR_ARG, "batch out of range");
    int rc = pdflow::net_seed(n, int(nb), d_input, d_output);
    if (rc) return rc;
    return check_net_status(n);
}

int pdflow_net_gradients(pdflow_net* n, unsigned nb, const float* d_input, const float* d_label, float* grads,
                         float* loss)
{
    if (!n || !d_input || !d_label) return net_fail(PDFLOW_ERR_ARG, "null argument");
    if (nb == 0 || nb > n->max_batch) return net_fail(PDFLOW_ERR_ARG, "batch out of range");
    int rc = forward_full(n, int(nb), d_input);
    if (!rc) rc = loss_and_grad(n, int(nb), d_input, d_label, loss);
    if (!rc) rc = backward(n, int(nb));
    if (rc) return rc;
    rc = check_net_status(n);
    if (rc) return rc;
    if (grads) {
        // canonical layout: per conv, dW [cout][K] then db [cout]
        for (size_t i = 0; i < n->conv.size(); ++i) {
            const Conv& c = n->conv[i];
            std::vector<float> gt(size_t(c.K()) * c.cout_pad);
            NET_TRY(cudaMemcpyAsync(gt.data(), n->gT[i], sizeof(float) * gt.size(), cudaMemcpyDeviceToHost,
                                    n->stream),
                    "D2H grads");
            NET_TRY(cudaMemcpyAsync(grads + c.boff, n->grad + c.boff, sizeof(float) * c.cout, cudaMemcpyDeviceToHost,
                                    n->stream),
                    "D2H grads");
            NET_TRY(cudaStreamSynchronize(n->stream), "synchronize");
            for (int o = 0; o < c.cout; ++o)
                for (int k = 0; k < c.K(); ++k) grads[c.woff + size_t(o) * c.K() + k] = gt[size_t(k) * c.cout_pad + o];
        }
    }
    return PDFLOW_OK;
}

int pdflow_net_train_step(pdflow_net* n, unsigned nb, const float* d_input, const float* d_label, float lr,
                          float* loss)
{
    if (!n || !d_input || !d_label) return net_fail(PDFLOW_ERR_ARG, "null argument");
    if (nb == 0 || nb > n->max_batch) return net_fail(PDFLOW_ERR_ARG, "batch out of range");
    if (!(lr > 0.f)) return net_fail(PDFLOW_ERR_ARG, "learning rate must be positive");
    int rc = forward_full(n, int(nb), d_input);
    if (!rc) rc = loss_and_grad(n, int(nb), d_input, d_label, loss);
    if (!rc) rc = backward(n, int(nb));
    if (rc) return rc;
    ++n->step;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - std::pow(b1, float(n->step)), c2 = 1.f - std::pow(b2, float(n->step));
    for (size_t i = 0; i < n->conv.size(); ++i) {
        const Conv& c = n->conv[i];
        k_adam_w<<<blocks(size_t(c.cout) * c.K()), 256, 0, n->stream>>>(
            n->w + c.woff, n->m + c.woff, n->v + c.woff, n->gT[i], c.cout, c.cout_pad, c.K(), lr, b1, b2, eps, c1, c2,
            1, n->Wb[i], n->WTb[i]);
        k_adam_b<<<blocks(size_t(c.cout)), 256, 0, n->stream>>>(n->w + c.boff, n->m + c.boff, n->v + c.boff,
                                                                  n->grad + c.boff, c.cout, lr, b1, b2, eps, c1, c2);
        NET_TRY(cudaGetLastError(), "adam launch");
    }
    return check_net_status(n);
}

int pdflow_gemm_bf16(int M, int N, int K, const void* d_a, int lda, const void* d_b, int ldb, float* d_c, int ldc,
                     int k_per_split, void* stream)
{
    if (!d_a || !d_b || !d_c) return net_fail(PDFLOW_ERR_ARG, "null argument");
    NET_TRY(prepare_gemm_once(), "GEMM kernel attributes");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned splits = k_per_split > 0 ? gemm_splits(K, k_per_split) : 1u;
    float* part = nullptr;
    unsigned* status = nullptr;
    NET_TRY(cudaMalloc(&status, sizeof(unsigned)), "status allocation");
    NET_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st), "status reset");
    if (splits > 1) NET_TRY(cudaMalloc(&part, sizeof(float) * size_t(splits) * M * ldc), "split-K allocation");
    GemmArgs g;
    g.A = d_a;
    g.B = d_b;
    g.M = M;
    g.N = N;
    g.K = K;
    g.lda = lda;
    g.ldb = ldb;
    g.C = splits > 1 ? part : d_c;
    g.ldc = ldc;
    g.bn = N >= 128 ? 128 : ((N + 15) / 16) * 16;
    g.k_per_split = splits > 1 ? k_per_split : 0;
    g.split_stride = size_t(M) * ldc;
    g.status = status;
    cudaError_t e = launch_gemm_tc(g, st);
    if (e == cudaSuccess && splits > 1) e = launch_splitk_sum(part, int(splits), g.split_stride, M, N, ldc, d_c, st);
    unsigned s = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, status, sizeof s, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(part);
    cudaFree(status);
    if (e != cudaSuccess) return net_fail(PDFLOW_ERR_CUDA, "GEMM", e);
    if (s) return net_fail(PDFLOW_ERR_TIMEOUT, "a tensor-core GEMM's bounded wait gave up");
    return PDFLOW_OK;
}

}  // extern "C"
