// nsdg_surrogate.cu — the warm-start network: a stack of 3x3 convolutions on
// the cell grid, trained and evaluated on the GPU with BF16 tensor-core
// kernels accumulating in FP32.
//
// Layout: activations channels-last, bfloat16, [batch][y][x][C] with C a
// multiple of 16; layer weights W[co][tap * Cin + ci] (tap = 3*dy + dx) in
// bfloat16 for the products, with FP32 master weights for Adam.  The
// convolution is an implicit GEMM (no im2col buffer): M = pixels, N = output
// channels, K = 9 * Cin; each K step (one tap, 16 input channels) is staged in
// shared memory with 16-byte loads and consumed by mma.sync m16n8k16
// (bf16 x bf16 -> f32).
//
// Network (matches oracle/cnn_oracle.py):
//   z_l = conv3x3(x_l, W_l) + b_l,  x_{l+1} = relu(z_l), identity after the last layer;
//   loss = sum m (out - target)^2 / (sum m * C_used).
// The weight gradient sums over pixels in fixed-size chunks (one block per
// chunk and tap) and the chunks are added in a fixed order, so training is
// deterministic.
#include "nsdg.h"
#include "nsdg_surrogate.hpp"

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace nsdg {

namespace {

constexpr int kBM = 64;       // pixels per GEMM block (4 warps x 16)
constexpr int kThreads = 128;
constexpr int kChunk = 2048;  // pixels per weight-gradient block
constexpr int kStride = 24;   // shared-memory row stride (16 + 8 halves): conflict-free fragments

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, const uint32_t* b)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

enum ConvMode { CONV_FWD_RELU = 0, CONV_FWD_LINEAR = 1, CONV_BWD_DATA = 2 };

// out[m][n] for m in a block of 64 pixels and all N channels.
//   forward:   A[m][(tap,c)] = src[pixel m + (dy-1, dx-1)][c],   B = W  [n][tap*CS + c]
//   bwd data:  A[m][(tap,c)] = src[pixel m - (dy-1, dx-1)][c],   B = W^T[n][tap*CS + c]
// CS = channels of src, N = channels of out.
template <int CS, int N, int MODE>
__global__ void __launch_bounds__(kThreads) kConv3x3(int B, int H, int W, const __nv_bfloat16* __restrict__ src,
    const __nv_bfloat16* __restrict__ wmat, const float* __restrict__ bias, const __nv_bfloat16* __restrict__ reluMask,
    __nv_bfloat16* __restrict__ outBf, float* __restrict__ outF)
{
    static_assert(CS % 16 == 0 && N % 8 == 0 && N <= 64, "channel counts");
    __shared__ __align__(16) __nv_bfloat16 As[kBM][kStride];
    __shared__ __align__(16) __nv_bfloat16 Bs[N][kStride];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t4 = lane & 3;
    const long M = long(B) * H * W;
    const long m0 = long(blockIdx.x) * kBM;
    // the pixel this thread loads for the A tile
    const int lm = tid >> 1, half = tid & 1;
    const long pm = m0 + lm;
    int pb = 0, py = 0, px = 0;
    const bool pvalid = pm < M;
    if (pvalid) {
        pb = static_cast<int>(pm / (long(H) * W));
        const int rem = static_cast<int>(pm - long(pb) * H * W);
        py = rem / W;
        px = rem % W;
    }
    float acc[N / 8][4];
#pragma unroll
    for (int j = 0; j < N / 8; ++j)
        acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int sgn = (MODE == CONV_BWD_DATA) ? -1 : 1;
    for (int tap = 0; tap < 9; ++tap) {
        const int oy = sgn * (tap / 3 - 1), ox = sgn * (tap % 3 - 1);
        const int sy = py + oy, sx = px + ox;
        const bool inside = pvalid && sy >= 0 && sy < H && sx >= 0 && sx < W;
        const __nv_bfloat16* srow = src + ((long(pb) * H + sy) * W + sx) * CS;
        for (int c0 = 0; c0 < CS; c0 += 16) {
            uint4 av = make_uint4(0, 0, 0, 0);
            if (inside)
                av = *reinterpret_cast<const uint4*>(srow + c0 + half * 8);
            *reinterpret_cast<uint4*>(&As[lm][half * 8]) = av;
            if (tid < 2 * N) {
                const int n = tid >> 1, hb = tid & 1;
                *reinterpret_cast<uint4*>(&Bs[n][hb * 8])
                    = *reinterpret_cast<const uint4*>(wmat + long(n) * 9 * CS + tap * CS + c0 + hb * 8);
            }
            __syncthreads();
            uint32_t a[4];
            const int r0 = warp * 16 + g;
            a[0] = *reinterpret_cast<const uint32_t*>(&As[r0][2 * t4]);
            a[1] = *reinterpret_cast<const uint32_t*>(&As[r0 + 8][2 * t4]);
            a[2] = *reinterpret_cast<const uint32_t*>(&As[r0][2 * t4 + 8]);
            a[3] = *reinterpret_cast<const uint32_t*>(&As[r0 + 8][2 * t4 + 8]);
#pragma unroll
            for (int j = 0; j < N / 8; ++j) {
                uint32_t b[2];
                b[0] = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + g][2 * t4]);
                b[1] = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + g][2 * t4 + 8]);
                mma16816(acc[j], a, b);
            }
            __syncthreads();
        }
    }
    // epilogue: rows warp*16 + g (+8), columns j*8 + 2*t4 (+1)
#pragma unroll
    for (int hrow = 0; hrow < 2; ++hrow) {
        const long m = m0 + warp * 16 + g + 8 * hrow;
        if (m >= M)
            continue;
#pragma unroll
        for (int j = 0; j < N / 8; ++j) {
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int n = j * 8 + 2 * t4 + cc;
                float v = acc[j][2 * hrow + cc];
                if (MODE == CONV_FWD_RELU) {
                    v = fmaxf(v + bias[n], 0.f);
                    outBf[m * N + n] = __float2bfloat16_rn(v);
                } else if (MODE == CONV_FWD_LINEAR) {
                    outF[m * N + n] = v + bias[n];
                } else {
                    // gradient w.r.t. the layer input, times relu'(previous pre-activation)
                    const float mk = __bfloat162float(reluMask[m * N + n]) > 0.f ? 1.f : 0.f;
                    outBf[m * N + n] = __float2bfloat16_rn(v * mk);
                }
            }
        }
    }
}

// Partial weight gradient of one tap over one chunk of pixels:
//   part[chunk][co][tap*CI + ci] = sum_{m in chunk} gz[m][co] * x[m + (dy-1, dx-1)][ci]
template <int CO, int CI>
__global__ void __launch_bounds__(kThreads) kConvWeightGrad(int B, int H, int W, const __nv_bfloat16* __restrict__ gz,
    const __nv_bfloat16* __restrict__ x, float* __restrict__ part)
{
    static_assert(CO % 16 == 0 && CI % 8 == 0 && CI <= 64 && CO <= 64, "channel counts");
    __shared__ __align__(16) __nv_bfloat16 As[CO][kStride]; // [co][pixel]
    __shared__ __align__(16) __nv_bfloat16 Bs[CI][kStride]; // [ci][pixel]
    const int tap = blockIdx.y, chunk = blockIdx.x;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t4 = lane & 3;
    const long M = long(B) * H * W;
    const long p0 = long(chunk) * kChunk;
    constexpr int NT = CI / 8, MT = CO / 16;
    constexpr int NTW = (NT + 3) / 4; // n8 tiles per warp (round robin)
    float acc[MT][NTW][4];
#pragma unroll
    for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int j = 0; j < NTW; ++j)
            acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
    for (int k0 = 0; k0 < kChunk; k0 += 16) {
        // A tile: 16 pixels x CO channels of gz, transposed into [co][pixel]
        for (int idx = tid; idx < 16 * (CO / 8); idx += kThreads) {
            const int pk = idx / (CO / 8), c8 = idx % (CO / 8);
            const long m = p0 + k0 + pk;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (m < M)
                v = *reinterpret_cast<const uint4*>(gz + m * CO + c8 * 8);
            const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
            for (int i = 0; i < 8; ++i)
                As[c8 * 8 + i][pk] = e[i];
        }
        // B tile: 16 pixels x CI channels of x at the shifted pixel, transposed into [ci][pixel]
        for (int idx = tid; idx < 16 * (CI / 8); idx += kThreads) {
            const int pk = idx / (CI / 8), c8 = idx % (CI / 8);
            const long m = p0 + k0 + pk;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (m < M) {
                const int b = static_cast<int>(m / (long(H) * W));
                const int rem = static_cast<int>(m - long(b) * H * W);
                const int sy = rem / W + dy, sx = rem % W + dx;
                if (sy >= 0 && sy < H && sx >= 0 && sx < W)
                    v = *reinterpret_cast<const uint4*>(x + ((long(b) * H + sy) * W + sx) * CI + c8 * 8);
            }
            const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
            for (int i = 0; i < 8; ++i)
                Bs[c8 * 8 + i][pk] = e[i];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < MT; ++i) {
            uint32_t a[4];
            const int r0 = i * 16 + g;
            a[0] = *reinterpret_cast<const uint32_t*>(&As[r0][2 * t4]);
            a[1] = *reinterpret_cast<const uint32_t*>(&As[r0 + 8][2 * t4]);
            a[2] = *reinterpret_cast<const uint32_t*>(&As[r0][2 * t4 + 8]);
            a[3] = *reinterpret_cast<const uint32_t*>(&As[r0 + 8][2 * t4 + 8]);
#pragma unroll
            for (int jj = 0; jj < NTW; ++jj) {
                const int j = warp + 4 * jj;
                if (j < NT) {
                    uint32_t b[2];
                    b[0] = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + g][2 * t4]);
                    b[1] = *reinterpret_cast<const uint32_t*>(&Bs[j * 8 + g][2 * t4 + 8]);
                    mma16816(acc[i][jj], a, b);
                }
            }
        }
        __syncthreads();
    }
    float* out = part + long(chunk) * CO * 9 * CI;
#pragma unroll
    for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int jj = 0; jj < NTW; ++jj) {
            const int j = warp + 4 * jj;
            if (j >= NT)
                continue;
#pragma unroll
            for (int hrow = 0; hrow < 2; ++hrow)
#pragma unroll
                for (int cc = 0; cc < 2; ++cc) {
                    const int co = i * 16 + g + 8 * hrow, ci = j * 8 + 2 * t4 + cc;
                    out[long(co) * 9 * CI + tap * CI + ci] = acc[i][jj][2 * hrow + cc];
                }
        }
}

// Sum of the chunk partials in chunk order (weight gradient), and the bias
// gradient from per-chunk channel sums.
__global__ void kSumChunks(int nChunks, size_t n, const float* __restrict__ part, float* __restrict__ out)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    float s = 0.f;
    for (int c = 0; c < nChunks; ++c)
        s += part[size_t(c) * n + i];
    out[i] = s;
}
template <int CO>
__global__ void kBiasGradPartial(long M, const __nv_bfloat16* __restrict__ gz, float* __restrict__ part)
{
    // one block per chunk, one thread per channel (blockDim.x = CO)
    const int co = threadIdx.x;
    const long p0 = long(blockIdx.x) * kChunk;
    float s = 0.f;
    for (int k = 0; k < kChunk; ++k) {
        const long m = p0 + k;
        if (m >= M)
            break;
        s += __bfloat162float(gz[m * CO + co]);
    }
    part[long(blockIdx.x) * CO + co] = s;
}

// Masked MSE: gz = 2 m (out - target) / denom for the first `used` channels
// (BF16, zero in the padding), per-block partial losses.
__global__ void __launch_bounds__(256) kLoss(long M, int C, int used, const float* __restrict__ out,
    const float* __restrict__ target, const float* __restrict__ mask, float invDenom, __nv_bfloat16* __restrict__ gz,
    float* __restrict__ partial)
{
    __shared__ float ws[8];
    const long m = blockIdx.x * long(blockDim.x) + threadIdx.x;
    float s = 0.f;
    if (m < M) {
        const float mk = mask[m];
        for (int c = 0; c < C; ++c) {
            float gval = 0.f;
            if (c < used) {
                const float d = out[m * C + c] - target[m * C + c];
                s += mk * d * d;
                gval = 2.f * mk * d * invDenom;
            }
            gz[m * C + c] = __float2bfloat16_rn(gval);
        }
    }
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w)
            t += ws[w];
        partial[blockIdx.x] = t * invDenom;
    }
}

__global__ void kAdam(size_t n, float* __restrict__ w, const float* __restrict__ gw, float* __restrict__ m1,
    float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const float gr = gw[i];
    const float a = b1 * m1[i] + (1.f - b1) * gr;
    const float b = b2 * m2[i] + (1.f - b2) * gr * gr;
    m1[i] = a;
    m2[i] = b;
    w[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// BF16 copies of one layer's weights: W [co][tap*CI+ci] and its transpose
// for the data gradient, WT [ci][tap*CO+co].
__global__ void kRefreshWeights(int CO, int CI, const float* __restrict__ w32, __nv_bfloat16* __restrict__ w16,
    __nv_bfloat16* __restrict__ wt16)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = CO * 9 * CI;
    if (i >= n)
        return;
    const int co = i / (9 * CI), rem = i % (9 * CI), tap = rem / CI, ci = rem % CI;
    const __nv_bfloat16 v = __float2bfloat16_rn(w32[i]);
    w16[i] = v;
    wt16[long(ci) * 9 * CO + tap * CO + co] = v;
}

__global__ void kToBf16(long n, const float* __restrict__ a, __nv_bfloat16* __restrict__ b)
{
    const long i = blockIdx.x * long(blockDim.x) + threadIdx.x;
    if (i < n)
        b[i] = __float2bfloat16_rn(a[i]);
}

template <int CS, int N, int MODE>
cudaError_t conv(cudaStream_t s, int B, int H, int W, const __nv_bfloat16* src, const __nv_bfloat16* w,
    const float* bias, const __nv_bfloat16* mask, __nv_bfloat16* outBf, float* outF)
{
    const long M = long(B) * H * W;
    const unsigned grid = static_cast<unsigned>((M + kBM - 1) / kBM);
    kConv3x3<CS, N, MODE><<<grid, kThreads, 0, s>>>(B, H, W, src, w, bias, mask, outBf, outF);
    return cudaGetLastError();
}

// channel counts supported by the instantiations: 16, 32, 48
#define NSDG_CH_SWITCH(c, D, CALL)                                                                 \
    switch (c) {                                                                                   \
    case 16: { constexpr int D = 16; CALL; } break;                                                \
    case 32: { constexpr int D = 32; CALL; } break;                                                \
    case 48: { constexpr int D = 48; CALL; } break;                                                \
    default: return cudaErrorInvalidValue;                                                         \
    }

} // namespace

// ---------------------------------------------------------------------------
// Network object
// ---------------------------------------------------------------------------
struct NetImpl {
    int L = 0;
    std::vector<int> ch;  // L+1 channel counts
    int H = 0, W = 0, maxB = 0, used = 0;
    cudaStream_t stream = nullptr;
    void* mem = nullptr;
    std::vector<size_t> wOff, bOff; // offsets into the FP32 parameter vector
    size_t nParams = 0;
    float *w32 = nullptr, *g32 = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *w16 = nullptr, *wt16 = nullptr;
    std::vector<__nv_bfloat16*> act; // L+1 bf16 activations (act[0] = input); act[L] unused
    float* out = nullptr;            // FP32 output [B][H][W][ch[L]]
    float* target = nullptr;
    float* mask = nullptr;
    __nv_bfloat16 *gA = nullptr, *gB = nullptr; // gradient ping-pong buffers
    float* part = nullptr;                       // chunk partials
    float* lossPart = nullptr;
    size_t partFloats = 0;
    int adamStep = 0;
    std::string err;
};

namespace {
size_t a256(size_t b) { return ((b + 255) / 256) * 256; }
}

int netCreate(int L, const int* channels, int H, int W, int maxB, int used, unsigned long long seed, NetImpl** out,
    std::string& err)
{
    if (L < 1 || L > 16 || H < 1 || W < 1 || maxB < 1) {
        err = "bad network shape";
        return NSDG_ERR_BAD_ARG;
    }
    for (int l = 0; l <= L; ++l)
        if (channels[l] != 16 && channels[l] != 32 && channels[l] != 48) {
            err = "channel counts must be 16, 32 or 48";
            return NSDG_ERR_BAD_ARG;
        }
    if (used < 1 || used > channels[L]) {
        err = "bad number of used output channels";
        return NSDG_ERR_BAD_ARG;
    }
    NetImpl* n = new NetImpl();
    n->L = L;
    n->ch.assign(channels, channels + L + 1);
    n->H = H;
    n->W = W;
    n->maxB = maxB;
    n->used = used;
    size_t off = 0;
    for (int l = 0; l < L; ++l) {
        n->wOff.push_back(off);
        off += size_t(n->ch[l + 1]) * 9 * n->ch[l];
        n->bOff.push_back(off);
        off += n->ch[l + 1];
    }
    n->nParams = off;
    const long M = long(maxB) * H * W;
    int cmax = 0;
    for (int c : n->ch)
        cmax = std::max(cmax, c);
    const long nChunks = (M + kChunk - 1) / kChunk;
    size_t wmax = 0;
    for (int l = 0; l < L; ++l)
        wmax = std::max(wmax, size_t(n->ch[l + 1]) * 9 * n->ch[l]);
    n->partFloats = size_t(nChunks) * wmax;
    size_t bytes = 4 * a256(n->nParams * 4) + 2 * a256(n->nParams * 2);
    for (int l = 0; l < L; ++l)
        bytes += a256(size_t(M) * n->ch[l] * 2);
    bytes += 2 * a256(size_t(M) * n->ch[L] * 4) + a256(size_t(M) * 4) + 2 * a256(size_t(M) * cmax * 2)
        + a256(n->partFloats * 4) + a256(size_t((M + 255) / 256 + 1) * 4);
    if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess
        || cudaMalloc(&n->mem, bytes) != cudaSuccess) {
        err = "network: device allocation failed";
        if (n->stream)
            cudaStreamDestroy(n->stream);
        delete n;
        return NSDG_ERR_CUDA;
    }
    char* p = static_cast<char*>(n->mem);
    auto take = [&](size_t b) {
        void* q = p;
        p += a256(b);
        return q;
    };
    n->w32 = static_cast<float*>(take(n->nParams * 4));
    n->g32 = static_cast<float*>(take(n->nParams * 4));
    n->m1 = static_cast<float*>(take(n->nParams * 4));
    n->m2 = static_cast<float*>(take(n->nParams * 4));
    n->w16 = static_cast<__nv_bfloat16*>(take(n->nParams * 2));
    n->wt16 = static_cast<__nv_bfloat16*>(take(n->nParams * 2));
    for (int l = 0; l < L; ++l)
        n->act.push_back(static_cast<__nv_bfloat16*>(take(size_t(M) * n->ch[l] * 2)));
    n->out = static_cast<float*>(take(size_t(M) * n->ch[L] * 4));
    n->target = static_cast<float*>(take(size_t(M) * n->ch[L] * 4));
    n->mask = static_cast<float*>(take(size_t(M) * 4));
    n->gA = static_cast<__nv_bfloat16*>(take(size_t(M) * cmax * 2));
    n->gB = static_cast<__nv_bfloat16*>(take(size_t(M) * cmax * 2));
    n->part = static_cast<float*>(take(n->partFloats * 4));
    n->lossPart = static_cast<float*>(take(size_t((M + 255) / 256 + 1) * 4));
    // He-normal initial weights, zero biases (host RNG: reproducible)
    std::vector<float> w(n->nParams, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < L; ++l) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (9.f * n->ch[l])));
        const size_t cnt = size_t(n->ch[l + 1]) * 9 * n->ch[l];
        for (size_t i = 0; i < cnt; ++i)
            w[n->wOff[l] + i] = nd(rng);
    }
    cudaError_t e = cudaMemcpy(n->w32, w.data(), n->nParams * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(n->m1, 0, n->nParams * 4);
    if (e == cudaSuccess) e = cudaMemset(n->m2, 0, n->nParams * 4);
    if (e == cudaSuccess) e = cudaMemset(n->mask, 0, size_t(M) * 4);
    if (e == cudaSuccess) e = cudaMemset(n->target, 0, size_t(M) * n->ch[L] * 4);
    if (e == cudaSuccess) e = netRefresh(n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->stream);
    if (e != cudaSuccess) {
        err = std::string("network init: ") + cudaGetErrorString(e);
        netDestroy(n);
        return NSDG_ERR_CUDA;
    }
    *out = n;
    return NSDG_OK;
}

void netDestroy(NetImpl* n)
{
    if (!n)
        return;
    if (n->stream)
        cudaStreamSynchronize(n->stream);
    if (n->mem)
        cudaFree(n->mem);
    if (n->stream)
        cudaStreamDestroy(n->stream);
    delete n;
}

cudaError_t netRefresh(NetImpl* n)
{
    for (int l = 0; l < n->L; ++l) {
        const int CO = n->ch[l + 1], CI = n->ch[l];
        const int cnt = CO * 9 * CI;
        kRefreshWeights<<<(cnt + 255) / 256, 256, 0, n->stream>>>(CO, CI, n->w32 + n->wOff[l], n->w16 + n->wOff[l],
            n->wt16 + n->wOff[l]);
    }
    return cudaGetLastError();
}

cudaStream_t netStream(NetImpl* n) { return n->stream; }
__nv_bfloat16* netInput(NetImpl* n) { return n->act[0]; }
float* netOutput(NetImpl* n) { return n->out; }
float* netTarget(NetImpl* n) { return n->target; }
float* netMask(NetImpl* n) { return n->mask; }
int netChannels(NetImpl* n, int l) { return n->ch[l]; }
int netLayers(NetImpl* n) { return n->L; }
size_t netParamCount(NetImpl* n) { return n->nParams; }
float* netParams(NetImpl* n) { return n->w32; }
float* netGrads(NetImpl* n) { return n->g32; }

cudaError_t netForward(NetImpl* n, cudaStream_t s, int B)
{
    if (B < 1 || B > n->maxB)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaSuccess;
    for (int l = 0; l < n->L && e == cudaSuccess; ++l) {
        const int CI = n->ch[l], CO = n->ch[l + 1];
        const __nv_bfloat16* w = n->w16 + n->wOff[l];
        const float* b = n->w32 + n->bOff[l];
        if (l + 1 < n->L) {
            NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = conv<A, Bc, CONV_FWD_RELU>(s, B, n->H, n->W, n->act[l], w, b,
                                                         nullptr, n->act[l + 1], nullptr))));
        } else {
            NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = conv<A, Bc, CONV_FWD_LINEAR>(s, B, n->H, n->W, n->act[l], w,
                                                         b, nullptr, nullptr, n->out))));
        }
    }
    return e;
}

cudaError_t netLossBackward(NetImpl* n, int B, float* lossDev)
{
    cudaStream_t s = n->stream;
    const long M = long(B) * n->H * n->W;
    const int CL = n->ch[n->L];
    // denominator: sum of the mask times the used channels (host-side sum of the device mask)
    std::vector<float> hm(M);
    cudaError_t e = cudaMemcpyAsync(hm.data(), n->mask, M * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return e;
    double msum = 0;
    for (float v : hm)
        msum += v;
    const float invDenom = msum > 0 ? static_cast<float>(1.0 / (msum * n->used)) : 0.f;
    const unsigned lb = static_cast<unsigned>((M + 255) / 256);
    kLoss<<<lb, 256, 0, s>>>(M, CL, n->used, n->out, n->target, n->mask, invDenom, n->gA, n->lossPart);
    kSumChunks<<<1, 1, 0, s>>>(static_cast<int>(lb), 1, n->lossPart, lossDev);
    const int nChunks = static_cast<int>((M + kChunk - 1) / kChunk);
    __nv_bfloat16* gz = n->gA;
    __nv_bfloat16* gnext = n->gB;
    for (int l = n->L - 1; l >= 0 && e == cudaSuccess; --l) {
        const int CI = n->ch[l], CO = n->ch[l + 1];
        const size_t nw = size_t(CO) * 9 * CI;
        // weight gradient
        dim3 grid(nChunks, 9);
        NSDG_CH_SWITCH(CO, A, NSDG_CH_SWITCH(CI, Bc, (kConvWeightGrad<A, Bc><<<grid, kThreads, 0, s>>>(B, n->H, n->W, gz,
                                                          n->act[l], n->part))));
        kSumChunks<<<static_cast<unsigned>((nw + 255) / 256), 256, 0, s>>>(nChunks, nw, n->part, n->g32 + n->wOff[l]);
        // bias gradient
        NSDG_CH_SWITCH(CO, A, (kBiasGradPartial<A><<<nChunks, A, 0, s>>>(M, gz, n->part)));
        kSumChunks<<<1, CO, 0, s>>>(nChunks, CO, n->part, n->g32 + n->bOff[l]);
        // data gradient times relu' of the layer input (not needed for the network input)
        if (l > 0) {
            NSDG_CH_SWITCH(CO, A, NSDG_CH_SWITCH(CI, Bc, (e = conv<A, Bc, CONV_BWD_DATA>(s, B, n->H, n->W, gz,
                                                              n->wt16 + n->wOff[l], nullptr, n->act[l], gnext, nullptr))));
            std::swap(gz, gnext);
        }
        if (e == cudaSuccess)
            e = cudaGetLastError();
    }
    return e;
}

cudaError_t netAdam(NetImpl* n, float lr, float b1, float b2, float eps)
{
    ++n->adamStep;
    const float c1 = 1.f - std::pow(b1, static_cast<float>(n->adamStep));
    const float c2 = 1.f - std::pow(b2, static_cast<float>(n->adamStep));
    kAdam<<<static_cast<unsigned>((n->nParams + 255) / 256), 256, 0, n->stream>>>(n->nParams, n->w32, n->g32, n->m1,
        n->m2, lr, b1, b2, eps, c1, c2);
    return netRefresh(n);
}

cudaError_t netInputFromFloat(NetImpl* n, long count, const float* dev)
{
    kToBf16<<<static_cast<unsigned>((count + 255) / 256), 256, 0, n->stream>>>(count, dev, n->act[0]);
    return cudaGetLastError();
}

} // namespace nsdg

// ===========================================================================
// C ABI (nsdg_net_*)
// ===========================================================================
struct nsdg_net {
    nsdg::NetImpl* impl = nullptr;
    std::string err;
    float* staging = nullptr; // device FP32 staging for host inputs
    size_t stagingFloats = 0;
    float* lossDev = nullptr;
};

using namespace nsdg;

extern "C" {

int nsdg_net_create(int n_layers, const int* channels, int height, int width, int max_batch, int used_outputs,
    unsigned long long seed, nsdg_net** out)
{
    if (!out || !channels)
        return NSDG_ERR_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return NSDG_ERR_NO_DEVICE;
    }
    nsdg_net* h = new nsdg_net();
    const int st = netCreate(n_layers, channels, height, width, max_batch, used_outputs, seed, &h->impl, h->err);
    if (st != NSDG_OK) {
        delete h;
        return st;
    }
    int cmax = 0;
    for (int l = 0; l <= n_layers; ++l)
        cmax = std::max(cmax, channels[l]);
    h->stagingFloats = size_t(max_batch) * height * width * cmax;
    if (cudaMalloc(&h->staging, h->stagingFloats * 4 + 256) != cudaSuccess) {
        netDestroy(h->impl);
        delete h;
        return NSDG_ERR_CUDA;
    }
    h->lossDev = h->staging + h->stagingFloats;
    *out = h;
    return NSDG_OK;
}

int nsdg_net_destroy(nsdg_net* h)
{
    if (!h)
        return NSDG_ERR_BAD_ARG;
    netDestroy(h->impl);
    cudaFree(h->staging);
    delete h;
    return NSDG_OK;
}

const char* nsdg_net_last_error(const nsdg_net* h) { return h ? h->err.c_str() : "null handle"; }

int nsdg_net_param_count(nsdg_net* h, size_t* n)
{
    if (!h || !n)
        return NSDG_ERR_BAD_ARG;
    *n = netParamCount(h->impl);
    return NSDG_OK;
}

static int netCopy(nsdg_net* h, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind)
{
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, netStream(h->impl));
    if (e == cudaSuccess) e = cudaStreamSynchronize(netStream(h->impl));
    if (e != cudaSuccess) {
        h->err = cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
    return NSDG_OK;
}

int nsdg_net_get_params(nsdg_net* h, float* host, size_t n)
{
    if (!h || !host || n != netParamCount(h->impl))
        return NSDG_ERR_BAD_ARG;
    return netCopy(h, host, netParams(h->impl), n * 4, cudaMemcpyDeviceToHost);
}

int nsdg_net_set_params(nsdg_net* h, const float* host, size_t n)
{
    if (!h || !host || n != netParamCount(h->impl))
        return NSDG_ERR_BAD_ARG;
    int r = netCopy(h, netParams(h->impl), host, n * 4, cudaMemcpyHostToDevice);
    if (r)
        return r;
    cudaError_t e = netRefresh(h->impl);
    if (e == cudaSuccess) e = cudaStreamSynchronize(netStream(h->impl));
    return e == cudaSuccess ? NSDG_OK : NSDG_ERR_CUDA;
}

int nsdg_net_get_grads(nsdg_net* h, float* host, size_t n)
{
    if (!h || !host || n != netParamCount(h->impl))
        return NSDG_ERR_BAD_ARG;
    return netCopy(h, host, netGrads(h->impl), n * 4, cudaMemcpyDeviceToHost);
}

int nsdg_net_set_batch(nsdg_net* h, int batch, const float* input, const float* target, const float* mask)
{
    if (!h || !input || batch < 1)
        return NSDG_ERR_BAD_ARG;
    NetImpl* n = h->impl;
    if (batch > n->maxB)
        return NSDG_ERR_SIZE_MISMATCH;
    const long M = long(batch) * n->H * n->W;
    const long cin = M * n->ch[0];
    int r = netCopy(h, h->staging, input, cin * 4, cudaMemcpyHostToDevice);
    if (r)
        return r;
    if (netInputFromFloat(n, cin, h->staging) != cudaSuccess)
        return NSDG_ERR_CUDA;
    if (target) {
        r = netCopy(h, netTarget(n), target, M * n->ch[n->L] * 4, cudaMemcpyHostToDevice);
        if (r)
            return r;
    }
    if (mask)
        return netCopy(h, netMask(n), mask, M * 4, cudaMemcpyHostToDevice);
    return NSDG_OK;
}

int nsdg_net_forward(nsdg_net* h, int batch, float* out_host)
{
    if (!h || batch < 1)
        return NSDG_ERR_BAD_ARG;
    NetImpl* n = h->impl;
    cudaError_t e = netForward(n, netStream(n), batch);
    if (e != cudaSuccess) {
        h->err = cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
    if (out_host)
        return netCopy(h, out_host, netOutput(n), size_t(batch) * n->H * n->W * n->ch[n->L] * 4,
            cudaMemcpyDeviceToHost);
    return NSDG_OK;
}

int nsdg_net_loss_backward(nsdg_net* h, int batch, float* loss)
{
    if (!h || batch < 1 || batch > h->impl->maxB)
        return NSDG_ERR_BAD_ARG;
    cudaError_t e = netLossBackward(h->impl, batch, h->lossDev);
    if (e != cudaSuccess) {
        h->err = cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
    if (loss)
        return netCopy(h, loss, h->lossDev, 4, cudaMemcpyDeviceToHost);
    return NSDG_OK;
}

int nsdg_net_adam_step(nsdg_net* h, float lr, float beta1, float beta2, float eps)
{
    if (!h || !(lr > 0))
        return NSDG_ERR_BAD_ARG;
    cudaError_t e = netAdam(h->impl, lr, beta1, beta2, eps);
    if (e != cudaSuccess) {
        h->err = cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
    return NSDG_OK;
}

} // extern "C"
