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
#include "nsdg_kernels.hpp"
#include "nsdg_surrogate.hpp"
#include "nsdg_tma.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
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

// Offset of the 8 channels [8 c8, 8 c8 + 8) of pixel m (m = (b H + y) W + x)
// in a C-channel BF16 activation map: channels-last, m C + 8 c8 (wg = 0,
// the mma.sync convolutions), or channel-group-major [b H + y][c8][x][8]
// (wg = W, the tensor-core convolutions: one 8-channel group of a row of
// pixels is contiguous, so one TMA box of it is one contiguous run).
__host__ __device__ __forceinline__ long actChunk(long m, int c8, int C, int wg)
{
    if (wg == 0)
        return m * C + c8 * 8;
    const long r = m / wg;
    return ((r * (C >> 3) + c8) * wg + (m - r * wg)) * 8;
}

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

// ---------------------------------------------------------------------------
// The same convolutions on the fifth-generation tensor cores (tcgen05).
//
// One tile is 128 consecutive pixels of one image row (the MMA's M = 128, one
// pixel per TMEM lane); N = output channels; K = 9 taps x CS channels, in
// steps of 16 (tcgen05.mma kind::f16, BF16 x BF16 -> FP32 in TMEM).
// Operands are K-major in shared memory without swizzle, in 8 x 16-byte core
// matrices: pixels (A rows) and output channels (B rows) 16 bytes apart, so
// 8-row groups are 128 bytes apart (SBO) and one 8-channel group of all rows
// is one contiguous block (LBO = the block's size).
//   A: the input rows, each in one slot of a ring in shared memory: pixels
//      x0-1 ... x0+134 (136 pixels) of all channel groups, [group][pixel][8]
//      (2176 bytes per group; pixels and rows outside the image read as zero),
//      brought by one TMA copy per row: the activations are stored
//      channel-group-major (actChunk), which a 5-D box lays out in shared
//      memory exactly as the MMAs read it.  A block walks a vertical strip
//      of tiles (one 128-pixel column, rows y0 .. y1-1) top to bottom, so
//      each input row is copied once and serves the three tiles that need
//      it.  Tap (dy, dx) of row y is the slot of input row y + dy - 1 with
//      its descriptor's start moved by dx pixels (16 bytes): no im2col.  The
//      data gradient uses the mirrored taps (2-dy, 2-dx).
//   B: all 9 taps of the weights, staged once per block.
// Warp roles: lane 0 of warp 8 loads the rows and issues the MMAs; warps 0-7
// read the two TMEM accumulators and write the tile: warp w reads TMEM lanes
// 32 (w % 4) .. + 31 (the tile's pixels) and output channels of half w / 4,
// two warps per scheduler.  rowFull/rowEmpty barriers hand the slots
// between the TMA and the MMAs (a row is released by the commit after the
// last tile that reads it), accFull/accEmpty the accumulators between the
// MMAs and the epilogue.  Every wait is bounded (nsdg_tma.cuh); a wait that
// runs out sets err and stops the block, whose copies and MMAs still in
// flight are waited for (bounded) before the TMEM is freed.
constexpr int kTcM = 128;
constexpr int kTcSpan = 136;
constexpr int kTcEpiWarps = 8;
constexpr int kTcThreads = 32 * (kTcEpiWarps + 1);
constexpr int kTcMaxSlots = 8;
constexpr unsigned kTcRowBytes = kTcSpan * 16; // 17 x 128: every TMA destination 128-byte aligned
constexpr unsigned kTcCols = 128;              // TMEM columns: two accumulators of up to 64
constexpr unsigned kTcSmemMax = 232448;        // dynamic shared memory per block (227 KB)

template <int CS, int N>
struct TcLayout {
    static constexpr unsigned kGroups = CS / 8;
    static constexpr unsigned kBBytes = 9u * CS * N * 2u;
    static constexpr unsigned kSlotBytes = kGroups * kTcRowBytes; // one input row
    static constexpr unsigned kAOff = (kBBytes + 1023u) & ~1023u;
    static constexpr unsigned kFit = (kTcSmemMax - 1024u - 256u - kAOff) / kSlotBytes;
    static constexpr unsigned kSlots = kFit > unsigned(kTcMaxSlots) ? unsigned(kTcMaxSlots) : kFit;
    static constexpr unsigned kBarOff = kAOff + kSlots * kSlotBytes;
    static constexpr unsigned kSmem = kBarOff + 256u + 1024u; // barriers, TMEM address, base alignment
    static_assert(kSlots >= 4, "four row slots must fit");
};

__device__ __forceinline__ uint64_t ummaDesc(unsigned addr, unsigned lbo, unsigned sbo)
{
    // start, leading (K) and stride (M/N) byte offsets in 16-byte units;
    // bits 46-48 = 0b001; base offset 0; no swizzle (bits 61-63 = 0)
    return uint64_t((addr & 0x3FFFFu) >> 4) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16)
        | (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

template <int N>
__host__ __device__ constexpr uint32_t ummaIdescBf16()
{
    // D F32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both
    // K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(kTcM >> 4) << 24);
}

// input row y of image b, pixels x .. x + 135, all channel groups of the
// channel-group-major map [b][y][g][x][8]: in shared memory [g][pixel][8]
__device__ __forceinline__ void tmaLoadRow(void* dst, const CUtensorMap* map, int x, int y, int b, uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smemAddr(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(x), "r"(0), "r"(y), "r"(b), "r"(smemAddr(bar))
                 : "memory");
}

__device__ __forceinline__ void mbarArrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar)) : "memory");
}

__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, int accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                 "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ void ummaCommit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar))
                 : "memory");
}

__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                 "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i)
        v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmemLoad8(uint32_t taddr, float* v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; ++i)
        v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// The work of a block: strips (b, 128-pixel column xt, rows y0 .. y1-1),
// strip i = blockIdx.x + k gridDim.x; a column holds `ns` strips of `hs` rows.
struct TcStrip {
    int b, x0, y0, y1;
};
__device__ __forceinline__ TcStrip tcStrip(long i, int H, int tilesX, int hs, int ns)
{
    const long col = i / ns;
    const int st = static_cast<int>(i - col * ns);
    TcStrip s;
    s.b = static_cast<int>(col / tilesX);
    s.x0 = static_cast<int>(col - long(s.b) * tilesX) * kTcM;
    s.y0 = st * hs;
    s.y1 = min(H, s.y0 + hs);
    return s;
}

template <int CS, int N, int MODE>
__global__ void __launch_bounds__(kTcThreads, 1) kConv3x3Tc(const __grid_constant__ CUtensorMap srcMap, int B,
    int H, int W, int hs, int ns, const __nv_bfloat16* __restrict__ wmat, const float* __restrict__ bias,
    const __nv_bfloat16* __restrict__ reluMask, __nv_bfloat16* __restrict__ outBf, float* __restrict__ outF,
    int* __restrict__ err)
{
    static_assert(CS % 16 == 0 && N % 16 == 0 && N <= 64, "channel counts");
    using Lay = TcLayout<CS, N>;
    constexpr int S = static_cast<int>(Lay::kSlots);
    extern __shared__ __align__(16) unsigned char tcSmemRaw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tcSmemRaw) + 1023) & ~uintptr_t(1023));
    unsigned char* sB = sm;
    unsigned char* sA = sm + Lay::kAOff;
    uint64_t* rowFull = reinterpret_cast<uint64_t*>(sm + Lay::kBarOff); // [8] a row has landed
    uint64_t* rowEmpty = rowFull + kTcMaxSlots;                         // [8] its last tile's MMAs completed
    uint64_t* accFull = rowEmpty + kTcMaxSlots;                         // [2] an accumulator is ready
    uint64_t* accEmpty = accFull + 2;                                   // [2] ... has been read
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(accEmpty + 2);
    __shared__ volatile int abortFlag;
    __shared__ float sBias[N];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // the weights in the core-matrix layout: 8-channel group g (tap * CS / 8
    // + channel group) of output channel n at g * N * 16 + n * 16
    for (int i = tid; i < 9 * (CS / 8) * N; i += kTcThreads) {
        const int n = i % N, g = i / N;
        const int tap = g / (CS / 8), cg = g % (CS / 8);
        *reinterpret_cast<uint4*>(sB + size_t(g) * N * 16 + n * 16)
            = *reinterpret_cast<const uint4*>(wmat + size_t(n) * 9 * CS + tap * CS + cg * 8);
    }
    if (MODE != CONV_BWD_DATA)
        for (int n = tid; n < N; n += kTcThreads)
            sBias[n] = bias[n];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) {
        for (int i = 0; i < 2 * kTcMaxSlots + 2; ++i)
            mbarInit(rowFull + i, 1);
        mbarInit(accEmpty, kTcEpiWarps * 32);
        mbarInit(accEmpty + 1, kTcEpiWarps * 32);
        abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    const uint32_t tmem = *tmemSlot;

    const int tilesX = (W + kTcM - 1) / kTcM;
    const long strips = long(B) * tilesX * ns;

    if (warp == kTcEpiWarps) {
        if (lane == 0) {
            // ---- rows and MMAs --------------------------------------------
            const uint32_t idesc = ummaIdescBf16<N>();
            const unsigned aBase = smemAddr(sA);
            const uint64_t bDesc0 = ummaDesc(smemAddr(sB), N * 16, 128);
            int loadPar[kTcMaxSlots];
            for (int i = 0; i < kTcMaxSlots; ++i)
                loadPar[i] = -1; // phase parity of a slot's outstanding copy
            int lastAcc = -1, lastAccPar = 0;
            long rowSeq = 0, tileSeq = 0;
            bool ok = true;
            for (long si = blockIdx.x; si < strips && ok; si += gridDim.x) {
                const TcStrip sp = tcStrip(si, H, tilesX, hs, ns);
                const int nt = sp.y1 - sp.y0, nr = nt + 2;
                const long base = rowSeq;
                int next = 0; // rows of this strip issued (input rows y0 - 1 + r)
                auto issueUpTo = [&](int limit) {
                    for (; ok && next < nr && next < limit; ++next) {
                        const long q = base + next;
                        const int slot = static_cast<int>(q % S);
                        // the slot's previous row has been read by its last tile
                        ok = mbarWaitBounded(rowEmpty + slot, static_cast<unsigned>(((q / S) & 1) ^ 1));
                        if (!ok)
                            break;
                        mbarExpectTx(rowFull + slot, Lay::kSlotBytes);
                        tmaLoadRow(sA + slot * Lay::kSlotBytes, &srcMap, sp.x0 - 1, sp.y0 - 1 + next, sp.b,
                            rowFull + slot);
                        loadPar[slot] = static_cast<int>((q / S) & 1);
                    }
                };
                for (int t = 0; t < nt && ok; ++t, ++tileSeq) {
                    if (abortFlag) {
                        ok = false;
                        break;
                    }
                    issueUpTo(t + S - 1);
                    // the tile's three rows t, t+1, t+2 of the strip
                    int slot3[3];
                    for (int r = 0; r < 3 && ok; ++r) {
                        const long q = base + t + r;
                        slot3[r] = static_cast<int>(q % S);
                        ok = mbarWaitBounded(rowFull + slot3[r], static_cast<unsigned>((q / S) & 1));
                        if (ok)
                            loadPar[slot3[r]] = -1;
                    }
                    const int acc = static_cast<int>(tileSeq & 1);
                    // the accumulator's previous tile has been read (its first
                    // use passes: the barrier's preceding phase counts as done)
                    ok = ok && mbarWaitBounded(accEmpty + acc, static_cast<unsigned>(((tileSeq >> 1) & 1) ^ 1));
                    if (!ok)
                        break;
                    tcFenceAfter();
                    const uint32_t d = tmem + acc * 64;
                    // a descriptor's start field is the address / 16, so the
                    // operands of every tap and K step are the three rows'
                    // and the weights' descriptors plus constants
                    const uint64_t aRow[3] = { ummaDesc(aBase + slot3[0] * Lay::kSlotBytes, kTcRowBytes, 128),
                        ummaDesc(aBase + slot3[1] * Lay::kSlotBytes, kTcRowBytes, 128),
                        ummaDesc(aBase + slot3[2] * Lay::kSlotBytes, kTcRowBytes, 128) };
#pragma unroll
                    for (int tap = 0; tap < 9; ++tap) {
                        const int dy = tap / 3, dx = tap % 3;
                        const int rb = MODE == CONV_BWD_DATA ? 2 - dy : dy;
                        const int sh = MODE == CONV_BWD_DATA ? 2 - dx : dx;
#pragma unroll
                        for (int ks = 0; ks < CS / 16; ++ks) {
                            const uint64_t ad = aRow[rb] + uint64_t(sh + 2 * ks * (kTcRowBytes >> 4));
                            const uint64_t bd = bDesc0 + uint64_t((tap * (CS / 8) + 2 * ks) * N);
                            umma(d, ad, bd, idesc, (tap | ks) != 0);
                        }
                    }
                    ummaCommit(accFull + acc);
                    lastAcc = acc;
                    lastAccPar = static_cast<int>((tileSeq >> 1) & 1);
                    // row t is last read by tile t; the strip's last tile also
                    // releases its two lower rows
                    ummaCommit(rowEmpty + slot3[0]);
                    if (t == nt - 1) {
                        ummaCommit(rowEmpty + slot3[1]);
                        ummaCommit(rowEmpty + slot3[2]);
                    }
                }
                rowSeq += nr;
            }
            if (!ok) {
                atomicOr(err, 1);
                abortFlag = 1;
            }
            // nothing of this block may still be in flight when it leaves
            for (int slot = 0; slot < S; ++slot)
                if (loadPar[slot] >= 0)
                    mbarWaitBounded(rowFull + slot, static_cast<unsigned>(loadPar[slot]));
            if (lastAcc >= 0)
                mbarWaitBounded(accFull + lastAcc, static_cast<unsigned>(lastAccPar));
        }
    } else {
        // ---- epilogue: warp w holds pixels x0 + 32 (w % 4) + lane, output
        // channels [NH (w / 4), NH (w / 4 + 1)) ----------------------------
        constexpr int NH = N / 2;
        const int quarter = warp & 3, half = warp >> 2;
        long tileSeq = 0;
        bool go = true;
        for (long si = blockIdx.x; si < strips && go; si += gridDim.x) {
            const TcStrip sp = tcStrip(si, H, tilesX, hs, ns);
            for (int y = sp.y0; y < sp.y1; ++y, ++tileSeq) {
                if (__any_sync(0xffffffffu, abortFlag != 0)) {
                    go = false;
                    break;
                }
                const int acc = static_cast<int>(tileSeq & 1);
                const bool ready
                    = __all_sync(0xffffffffu, mbarWaitBounded(accFull + acc, static_cast<unsigned>((tileSeq >> 1) & 1)));
                if (!ready) {
                    if (lane == 0) {
                        atomicOr(err, 1);
                        abortFlag = 1;
                    }
                    go = false;
                    break;
                }
                tcFenceAfter();
                float v[NH];
                const uint32_t taddr = tmem + acc * 64 + half * NH + (uint32_t(32 * quarter) << 16);
#pragma unroll
                for (int c = 0; c < NH; c += 8)
                    tmemLoad8(taddr + c, v + c);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                tcFenceBefore();
                mbarArrive(accEmpty + acc);
                const int x = sp.x0 + 32 * quarter + lane;
                if (x < W) {
                    const long row = long(sp.b) * H + y;
                    const int n0 = half * NH;
                    if (MODE == CONV_FWD_LINEAR) {
                        const long m = row * W + x;
#pragma unroll
                        for (int c = 0; c < NH; c += 4) {
                            const int n = n0 + c;
                            *reinterpret_cast<float4*>(outF + m * N + n) = make_float4(v[c] + sBias[n],
                                v[c + 1] + sBias[n + 1], v[c + 2] + sBias[n + 2], v[c + 3] + sBias[n + 3]);
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < NH; c += 8) {
                            const int n = n0 + c;
                            // actChunk of pixel (row, x): the row is known
                            const long off = ((row * (N >> 3) + (n >> 3)) * W + x) * 8;
                            uint4 mk4 = make_uint4(0, 0, 0, 0);
                            if (MODE == CONV_BWD_DATA)
                                mk4 = *reinterpret_cast<const uint4*>(reluMask + off);
                            const __nv_bfloat16* mk = reinterpret_cast<const __nv_bfloat16*>(&mk4);
                            __nv_bfloat16 o[8];
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                float val = v[c + j];
                                if (MODE == CONV_FWD_RELU)
                                    val = fmaxf(val + sBias[n + j], 0.f);
                                else
                                    val = __bfloat162float(mk[j]) > 0.f ? val : 0.f;
                                o[j] = __float2bfloat16_rn(val);
                            }
                            *reinterpret_cast<uint4*>(outBf + off) = *reinterpret_cast<const uint4*>(o);
                        }
                    }
                }
            }
        }
    }
    tcFenceBefore();
    __syncthreads();
    if (warp == 0) {
        tcFenceAfter();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
    }
}

// ---------------------------------------------------------------------------
// The weight gradient on the tensor cores:
//   part[blk][co][tap*CI + ci] = sum over the block's pixels p of
//                                x[p + (dy-1, dx-1)][ci] gz[p][co]
// One MMA: M = 128 rows of input channels (rows CI .. 127 read whatever lies
// beyond the row in shared memory and are discarded), N = CO, K = 16 pixels.
// Both operands are MN-major and come straight from the channel-group-major
// rows ([g][pixel][8]: 8 channels of one pixel in 16 bytes), no transposes:
//   A: the input row y + dy - 1 in a ring slot (pixels x0-1 .. x0+134, the
//      forward kernel's rows), start moved by dx pixels; 8-channel groups
//      2176 bytes apart (SBO), 8-pixel groups 128 bytes apart (LBO);
//   B: gz row y, pixels x0 .. x0+127, one TMA copy into one of two buffers;
//      groups 2048 bytes apart, 8-pixel groups 128 bytes apart.
// Nine accumulators (one per tap) of CO columns stay in TMEM while the block
// walks its strips (each a 128-pixel column's rows y0 .. y1-1; each input row
// copied once and used by three rows of gz), and are read once at the end by
// warps 0-3 (TMEM lanes = input channels).  Lane 0 of warp 4 issues the
// copies and the MMAs.  Every wait is bounded; a wait that runs out sets err,
// and the block still waits (bounded) for its copies and MMAs in flight
// before it frees the TMEM.
constexpr int kWgThreads = 32 * 5;
constexpr unsigned kWgGzGroupBytes = kTcM * 16; // one 8-channel group of one gz row: 128 pixels

template <int CI, int CO, int MR>
struct WgLayout {
    static constexpr unsigned kSlotBytes = (CI / 8) * kTcRowBytes;
    static constexpr unsigned kGzBytes = (CO / 8) * kWgGzGroupBytes;
    static constexpr unsigned kAOff = (2 * kGzBytes + 1023u) & ~1023u;
    // the MR-row A operand of the last slot reads up to MR / 8 groups and
    // the largest shift and K step beyond the slot's start
    static constexpr unsigned kPad = (unsigned(MR / 8) - CI / 8) * kTcRowBytes + kTcRowBytes;
    static constexpr unsigned kFit = (kTcSmemMax - 1024u - 256u - kAOff - kPad) / kSlotBytes;
    static constexpr unsigned kSlots = kFit > unsigned(kTcMaxSlots) ? unsigned(kTcMaxSlots) : kFit;
    static constexpr unsigned kBarOff = kAOff + kSlots * kSlotBytes + kPad;
    static constexpr unsigned kSmem = kBarOff + 256u + 1024u;
    static_assert(kSlots >= 4, "four row slots must fit");
};

__device__ __forceinline__ void tmaLoadGzRow(void* dst, const CUtensorMap* map, int x, int y, int b, uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smemAddr(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(x), "r"(0), "r"(y), "r"(b), "r"(smemAddr(bar))
                 : "memory");
}

template <int CI, int CO, int MR>
__global__ void __launch_bounds__(kWgThreads, 1) kConvWeightGradTc(const __grid_constant__ CUtensorMap xMap,
    const __grid_constant__ CUtensorMap gzMap, int B, int H, int W, int hs, int ns, float* __restrict__ part,
    int* __restrict__ err)
{
    static_assert(CI % 8 == 0 && CI <= MR && (MR == 64 || MR == 128) && CO % 16 == 0 && 9 * CO <= 512,
        "channel counts");
    using Lay = WgLayout<CI, CO, MR>;
    constexpr int S = static_cast<int>(Lay::kSlots);
    constexpr uint32_t kCols = 512;
    extern __shared__ __align__(16) unsigned char wgSmemRaw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(wgSmemRaw) + 1023) & ~uintptr_t(1023));
    unsigned char* sGz = sm;
    unsigned char* sA = sm + Lay::kAOff;
    uint64_t* rowFull = reinterpret_cast<uint64_t*>(sm + Lay::kBarOff); // [8]
    uint64_t* rowEmpty = rowFull + kTcMaxSlots;                         // [8]
    uint64_t* gzFull = rowEmpty + kTcMaxSlots;                          // [2]
    uint64_t* gzEmpty = gzFull + 2;                                     // [2]
    uint64_t* done = gzEmpty + 2;                                       // [1] every MMA of the block completed
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(done + 1);
    __shared__ volatile int abortFlag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < 2 * kTcMaxSlots + 5; ++i)
            mbarInit(rowFull + i, 1);
        abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    const uint32_t tmem = *tmemSlot;
    const int tilesX = (W + kTcM - 1) / kTcM;
    const long strips = long(B) * tilesX * ns;

    if (warp == 4) {
        if (lane == 0) {
            // D F32, A and B BF16, both MN-major (bits 15, 16), N = CO, M = MR
            constexpr uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16)
                | (uint32_t(CO >> 3) << 17) | (uint32_t(MR >> 4) << 24);
            const unsigned aBase = smemAddr(sA);
            const uint64_t gzDesc[2] = { ummaDesc(smemAddr(sGz), 128, kWgGzGroupBytes),
                ummaDesc(smemAddr(sGz + Lay::kGzBytes), 128, kWgGzGroupBytes) };
            int loadPar[kTcMaxSlots];
            for (int i = 0; i < kTcMaxSlots; ++i)
                loadPar[i] = -1;
            int gzPar[2] = { -1, -1 };
            long rowSeq = 0, chunkSeq = 0;
            bool ok = true;
            for (long si = blockIdx.x; si < strips && ok; si += gridDim.x) {
                const TcStrip sp = tcStrip(si, H, tilesX, hs, ns);
                const int nt = sp.y1 - sp.y0, nr = nt + 2;
                const long base = rowSeq;
                int next = 0;
                auto issueUpTo = [&](int limit) {
                    for (; ok && next < nr && next < limit; ++next) {
                        const long q = base + next;
                        const int slot = static_cast<int>(q % S);
                        ok = mbarWaitBounded(rowEmpty + slot, static_cast<unsigned>(((q / S) & 1) ^ 1));
                        if (!ok)
                            break;
                        mbarExpectTx(rowFull + slot, Lay::kSlotBytes);
                        tmaLoadRow(sA + slot * Lay::kSlotBytes, &xMap, sp.x0 - 1, sp.y0 - 1 + next, sp.b,
                            rowFull + slot);
                        loadPar[slot] = static_cast<int>((q / S) & 1);
                    }
                };
                auto issueGz = [&](long c, int y) {
                    const int g = static_cast<int>(c & 1);
                    ok = ok && mbarWaitBounded(gzEmpty + g, static_cast<unsigned>(((c >> 1) & 1) ^ 1));
                    if (!ok)
                        return;
                    mbarExpectTx(gzFull + g, Lay::kGzBytes);
                    tmaLoadGzRow(sGz + g * Lay::kGzBytes, &gzMap, sp.x0, y, sp.b, gzFull + g);
                    gzPar[g] = static_cast<int>((c >> 1) & 1);
                };
                issueGz(chunkSeq, sp.y0);
                for (int t = 0; t < nt && ok; ++t, ++chunkSeq) {
                    if (t + 1 < nt)
                        issueGz(chunkSeq + 1, sp.y0 + t + 1);
                    issueUpTo(t + S - 1);
                    int slot3[3];
                    for (int r = 0; r < 3 && ok; ++r) {
                        const long q = base + t + r;
                        slot3[r] = static_cast<int>(q % S);
                        ok = mbarWaitBounded(rowFull + slot3[r], static_cast<unsigned>((q / S) & 1));
                        if (ok)
                            loadPar[slot3[r]] = -1;
                    }
                    const int g = static_cast<int>(chunkSeq & 1);
                    ok = ok && mbarWaitBounded(gzFull + g, static_cast<unsigned>((chunkSeq >> 1) & 1));
                    if (!ok)
                        break;
                    gzPar[g] = -1;
                    tcFenceAfter();
                    const uint64_t aRow[3] = { ummaDesc(aBase + slot3[0] * Lay::kSlotBytes, 128, kTcRowBytes),
                        ummaDesc(aBase + slot3[1] * Lay::kSlotBytes, 128, kTcRowBytes),
                        ummaDesc(aBase + slot3[2] * Lay::kSlotBytes, 128, kTcRowBytes) };
#pragma unroll
                    for (int tap = 0; tap < 9; ++tap) {
                        const int dy = tap / 3, dx = tap % 3;
#pragma unroll
                        for (int ks = 0; ks < kTcM / 16; ++ks)
                            umma(tmem + tap * CO, aRow[dy] + uint64_t(dx + 16 * ks), gzDesc[g] + uint64_t(16 * ks),
                                idesc, (chunkSeq > 0 || ks > 0) ? 1 : 0);
                    }
                    ummaCommit(gzEmpty + g);
                    ummaCommit(rowEmpty + slot3[0]);
                    if (t == nt - 1) {
                        ummaCommit(rowEmpty + slot3[1]);
                        ummaCommit(rowEmpty + slot3[2]);
                    }
                }
                rowSeq += nr;
            }
            if (!ok) {
                atomicOr(err, 1);
                abortFlag = 1;
            }
            ummaCommit(done); // arrives once every MMA issued above has completed
            for (int slot = 0; slot < S; ++slot)
                if (loadPar[slot] >= 0)
                    mbarWaitBounded(rowFull + slot, static_cast<unsigned>(loadPar[slot]));
            for (int g = 0; g < 2; ++g)
                if (gzPar[g] >= 0)
                    mbarWaitBounded(gzFull + g, static_cast<unsigned>(gzPar[g]));
        }
    } else {
        // warp w reads TMEM lanes 32 w .. 32 w + 31: input channel ci = 32 w +
        // lane for M = 128; for M = 64 the accumulator rows sit in the first
        // 16 lanes of each 32-lane quarter, ci = 16 w + lane (lane < 16)
        const bool ready = __all_sync(0xffffffffu, mbarWaitBounded(done, 0));
        if (!ready && lane == 0) {
            atomicOr(err, 1);
            abortFlag = 1;
        }
        if (ready && !abortFlag) {
            tcFenceAfter();
            const int ci = MR == 128 ? 32 * warp + lane : (lane < 16 ? 16 * warp + lane : CI);
            float* out = part + long(blockIdx.x) * CO * 9 * CI;
#pragma unroll 1
            for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
                for (int c = 0; c < CO; c += 8) {
                    float v[8];
                    tmemLoad8(tmem + tap * CO + c + (uint32_t(32 * warp) << 16), v);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (ci < CI) {
#pragma unroll
                        for (int j = 0; j < 8; ++j)
                            out[long(c + j) * 9 * CI + tap * CI + ci] = v[j];
                    }
                }
            }
        }
    }
    tcFenceBefore();
    __syncthreads();
    if (warp == 0) {
        tcFenceAfter();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

// Partial weight gradient of one tap over one chunk of pixels:
//   part[chunk][co][tap*CI + ci] = sum_{m in chunk} gz[m][co] * x[m + (dy-1, dx-1)][ci]
template <int CO, int CI>
__global__ void __launch_bounds__(kThreads) kConvWeightGrad(int B, int H, int W, const __nv_bfloat16* __restrict__ gz,
    const __nv_bfloat16* __restrict__ x, float* __restrict__ part, int wg)
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
                v = *reinterpret_cast<const uint4*>(gz + actChunk(m, c8, CO, wg));
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
                    v = *reinterpret_cast<const uint4*>(x + actChunk((long(b) * H + sy) * W + sx, c8, CI, wg));
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
// out[i] = sum over c < nParts of part[c * n + i], one block of 256 threads
// per output (for few outputs with many partials: the bias gradients, the loss)
__global__ void __launch_bounds__(256) kSumPartsBlock(int nParts, size_t n, const float* __restrict__ part,
    float* __restrict__ out)
{
    __shared__ float ws[8];
    const size_t i = blockIdx.x;
    float s = 0.f;
    for (int c = threadIdx.x; c < nParts; c += 256)
        s += part[size_t(c) * n + i];
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w)
            t += ws[w];
        out[i] = t;
    }
}

// Bias gradient partial of one chunk of kChunk pixels: part[chunk][co] =
// sum of gz[m][co]; 256 threads read one 8-channel group of consecutive
// pixels at a time (16 bytes each, coalesced), then reduce per channel.
template <int CO>
__global__ void __launch_bounds__(256) kBiasGradPartial(long M, const __nv_bfloat16* __restrict__ gz,
    float* __restrict__ part, int wg)
{
    __shared__ float red[8][8];
    const long p0 = long(blockIdx.x) * kChunk;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int g = 0; g < CO / 8; ++g) {
        float acc[8] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
        for (int k = tid; k < kChunk; k += 256) {
            const long m = p0 + k;
            if (m >= M)
                break;
            const uint4 v = *reinterpret_cast<const uint4*>(gz + actChunk(m, g, CO, wg));
            const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                acc[j] += __bfloat162float(e[j]);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            for (int off = 16; off > 0; off >>= 1)
                acc[j] += __shfl_down_sync(0xffffffffu, acc[j], off);
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < 8; ++j)
                red[warp][j] = acc[j];
        __syncthreads();
        if (tid < 8) {
            float t = 0.f;
            for (int w = 0; w < 8; ++w)
                t += red[w][tid];
            part[long(blockIdx.x) * CO + g * 8 + tid] = t;
        }
        __syncthreads();
    }
}

// Masked MSE: gz = 2 m (out - target) / denom for the first `used` channels
// (BF16, zero in the padding), per-block partial losses.
__global__ void __launch_bounds__(256) kLoss(long M, int C, int used, const float* __restrict__ out,
    const float* __restrict__ target, const float* __restrict__ mask, const float* __restrict__ invDenomPtr,
    __nv_bfloat16* __restrict__ gz, float* __restrict__ partial, int wg)
{
    __shared__ float ws[8];
    const float invDenom = *invDenomPtr;
    const long m = blockIdx.x * long(blockDim.x) + threadIdx.x;
    float s = 0.f;
    if (m < M) {
        const float mk = mask[m];
        // 8 channels at a time: two float4 of the output and of the target,
        // one 16-byte group of gz
        for (int g = 0; g < C / 8; ++g) {
            const float4* o4 = reinterpret_cast<const float4*>(out + m * C + g * 8);
            const float4* t4 = reinterpret_cast<const float4*>(target + m * C + g * 8);
            const float4 oa = o4[0], ob = o4[1], ta = t4[0], tb = t4[1];
            const float ov[8] = { oa.x, oa.y, oa.z, oa.w, ob.x, ob.y, ob.z, ob.w };
            const float tv[8] = { ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w };
            __align__(16) __nv_bfloat16 gv[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float gval = 0.f;
                if (g * 8 + j < used) {
                    const float d = ov[j] - tv[j];
                    s += mk * d * d;
                    gval = 2.f * mk * d * invDenom;
                }
                gv[j] = __float2bfloat16_rn(gval);
            }
            *reinterpret_cast<uint4*>(gz + actChunk(m, g, C, wg)) = *reinterpret_cast<const uint4*>(gv);
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

// 1 / (sum of the mask * used channels), one block, fixed summation order
// The loss denominator (sum of the mask times the used channels) in two
// passes: per-block sums of 256 mask values (exact in FP32 for a 0/1 mask),
// then one block adds them in FP64 and stores 1 / denominator.
__global__ void __launch_bounds__(256) kMaskPartial(long M, const float* __restrict__ mask,
    float* __restrict__ partial)
{
    __shared__ float ws[8];
    const long m = blockIdx.x * 256L + threadIdx.x;
    float s = m < M ? mask[m] : 0.f;
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w)
            t += ws[w];
        partial[blockIdx.x] = t;
    }
}
__global__ void __launch_bounds__(256) kInvDenom(int nPartial, int used, const float* __restrict__ partial,
    float* __restrict__ invDenom)
{
    __shared__ double ws[8];
    double s = 0.0;
    for (int i = threadIdx.x; i < nPartial; i += 256)
        s += partial[i];
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w)
            t += ws[w];
        *invDenom = t > 0.0 ? static_cast<float>(1.0 / (t * used)) : 0.f;
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

// channels-last FP32 input [M][C] -> the network's BF16 input map
__global__ void kToBf16(long n, int C, int wg, const float* __restrict__ a, __nv_bfloat16* __restrict__ b)
{
    const long i = blockIdx.x * long(blockDim.x) + threadIdx.x;
    if (i < n) {
        const long m = i / C;
        const int c = static_cast<int>(i - m * C);
        b[actChunk(m, c >> 3, C, wg) + (c & 7)] = __float2bfloat16_rn(a[i]);
    }
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

// The tensor-core form: a tensor map over the source [B][H][W][CS] (boxes of
// 8 channels x 136 pixels), one block per SM looping over the tiles.
template <int CS, int N, int MODE>
cudaError_t convTcPrepare()
{
    return cudaFuncSetAttribute(kConv3x3Tc<CS, N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        static_cast<int>(TcLayout<CS, N>::kSmem));
}

template <int CS, int N, int MODE>
cudaError_t convTc(cudaStream_t s, int B, int H, int W, const __nv_bfloat16* src, const __nv_bfloat16* w,
    const float* bias, const __nv_bfloat16* mask, __nv_bfloat16* outBf, float* outF, int* err)
{
    // the source [B][H][CS/8][W][8] (channel-group-major), boxes of 136
    // pixels x all channel groups of one row
    CUtensorMap map;
    const uint64_t dims[5] = { 8, uint64_t(W), uint64_t(CS / 8), uint64_t(H), uint64_t(B) };
    const uint64_t strides[4] = { 16, uint64_t(W) * 16, uint64_t(W) * CS * 2, uint64_t(H) * W * CS * 2 };
    const uint32_t box[5] = { 8, kTcSpan, uint32_t(CS / 8), 1, 1 };
    cudaError_t e = encodeTiledNd(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, src, 5, dims, strides, box);
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return e;
    // vertical strips: about one per SM, each a 128-pixel column's rows
    // y0 .. y0 + hs - 1
    const long columns = long(B) * ((W + kTcM - 1) / kTcM);
    const int want = static_cast<int>(std::max<long>(1, sms / columns));
    const int hs = (H + want - 1) / want;
    const int ns = (H + hs - 1) / hs;
    const unsigned grid = static_cast<unsigned>(std::min<long>(columns * ns, sms));
    kConv3x3Tc<CS, N, MODE><<<grid, kTcThreads, TcLayout<CS, N>::kSmem, s>>>(map, B, H, W, hs, ns, w, bias, mask,
        outBf, outF, err);
    return cudaGetLastError();
}

template <int CI, int CO>
cudaError_t convWeightGradTcPrepare()
{
    if constexpr (9 * CO > 512) {
        return cudaSuccess; // kept on mma.sync (nine accumulators of CO columns exceed the TMEM)
    } else {
        cudaError_t e = cudaFuncSetAttribute(kConvWeightGradTc<CI, CO, 128>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(WgLayout<CI, CO, 128>::kSmem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kConvWeightGradTc<CI, CO, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                static_cast<int>(WgLayout<CI, CO, 64>::kSmem));
        return e;
    }
}

// MMA rows of the weight gradient: 64 (input channels padded to 64, the
// default) or 128 (NSDG_WGRAD_M=128)
inline int wgradRows()
{
    const char* e = std::getenv("NSDG_WGRAD_M");
    return e && std::strcmp(e, "128") == 0 ? 128 : 64;
}

// The weight gradient's partial sums on the tensor cores into part[0 ..
// *nParts); maxParts bounds the partial buffer (in CO x 9 x CI sets).
template <int CI, int CO>
cudaError_t convWeightGradTc(cudaStream_t s, int B, int H, int W, const __nv_bfloat16* gz, const __nv_bfloat16* x,
    float* part, long maxParts, int* err, int* nParts)
{
    if constexpr (9 * CO > 512) {
        return cudaErrorNotSupported;
    } else {
        CUtensorMap xm, gm;
        const uint64_t xd[5] = { 8, uint64_t(W), uint64_t(CI / 8), uint64_t(H), uint64_t(B) };
        const uint64_t xs[4] = { 16, uint64_t(W) * 16, uint64_t(W) * CI * 2, uint64_t(H) * W * CI * 2 };
        const uint32_t xb[5] = { 8, kTcSpan, uint32_t(CI / 8), 1, 1 };
        const uint64_t gd[5] = { 8, uint64_t(W), uint64_t(CO / 8), uint64_t(H), uint64_t(B) };
        const uint64_t gs[4] = { 16, uint64_t(W) * 16, uint64_t(W) * CO * 2, uint64_t(H) * W * CO * 2 };
        const uint32_t gb[5] = { 8, uint32_t(kTcM), uint32_t(CO / 8), 1, 1 };
        cudaError_t e = encodeTiledNd(&xm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, x, 5, xd, xs, xb);
        if (e == cudaSuccess) e = encodeTiledNd(&gm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, gz, 5, gd, gs, gb);
        int dev = 0, sms = 0;
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return e;
        // one block per SM at most, no more blocks than partial sets; each
        // block's strips as tall as that allows
        const long columns = long(B) * ((W + kTcM - 1) / kTcM);
        const long cap = std::max<long>(1, std::min<long>(sms, maxParts));
        const int want = static_cast<int>(std::max<long>(1, cap / columns));
        const int hs = (H + want - 1) / want;
        const int ns = (H + hs - 1) / hs;
        const unsigned grid = static_cast<unsigned>(std::min<long>(columns * ns, cap));
        if (wgradRows() == 128)
            kConvWeightGradTc<CI, CO, 128><<<grid, kWgThreads, WgLayout<CI, CO, 128>::kSmem, s>>>(xm, gm, B, H, W, hs,
                ns, part, err);
        else
            kConvWeightGradTc<CI, CO, 64><<<grid, kWgThreads, WgLayout<CI, CO, 64>::kSmem, s>>>(xm, gm, B, H, W, hs,
                ns, part, err);
        *nParts = static_cast<int>(grid);
        return cudaGetLastError();
    }
}

// channel counts supported by the instantiations: 16, 32, 48, 64
#define NSDG_CH_SWITCH(c, D, CALL)                                                                 \
    switch (c) {                                                                                   \
    case 16: { constexpr int D = 16; CALL; } break;                                                \
    case 32: { constexpr int D = 32; CALL; } break;                                                \
    case 48: { constexpr int D = 48; CALL; } break;                                                \
    case 64: { constexpr int D = 64; CALL; } break;                                                \
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
    // dataset (raw FP32) and normalisation
    void* dsMem = nullptr;
    int dsCap = 0;
    float *dsX = nullptr, *dsY = nullptr, *dsM = nullptr;
    float* stats = nullptr; // device: featShift[kWarmFeat], featInv[kWarmFeat], tgtShift[kWarmTgt], tgtScale[kWarmTgt]
    int* dIdx = nullptr;    // batch sample indices
    double* dPart = nullptr;
    // convolutions on tcgen05 (the default) or by mma.sync (NSDG_CONV=mma);
    // the tensor-core kernels' error word (a bounded wait ran out)
    bool tc = true;
    int wg = 0; // activation layout: 0 channels-last, W channel-group-major (tc)
    int* derr = nullptr;
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
        if (channels[l] != 16 && channels[l] != 32 && channels[l] != 48 && channels[l] != 64) {
            err = "channel counts must be 16, 32, 48 or 64";
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
    size_t bytes = 4 * a256(n->nParams * 4) + 2 * a256(n->nParams * 2) + a256(kWarmNorm * 4)
        + a256(size_t(maxB) * 4);
    for (int l = 0; l < L; ++l)
        bytes += a256(size_t(M) * n->ch[l] * 2);
    bytes += 2 * a256(size_t(M) * n->ch[L] * 4) + a256(size_t(M) * 4) + 2 * a256(size_t(M) * cmax * 2)
        + a256(n->partFloats * 4) + a256(size_t((M + 255) / 256 + 2) * 4) + a256(4);
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
    n->lossPart = static_cast<float*>(take(size_t((M + 255) / 256 + 2) * 4));
    n->stats = static_cast<float*>(take(kWarmNorm * 4));
    n->dIdx = static_cast<int*>(take(size_t(maxB) * 4));
    n->derr = static_cast<int*>(take(4));
    if (const char* env = std::getenv("NSDG_CONV"))
        n->tc = std::strcmp(env, "mma") != 0;
    n->wg = n->tc ? W : 0;
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
    if (e == cudaSuccess) e = cudaMemset(n->derr, 0, 4);
    // the tensor-core kernels' shared memory, once per instantiation used
    for (int l = 0; l < L && e == cudaSuccess && n->tc; ++l) {
        const int CI = n->ch[l], CO = n->ch[l + 1];
        const auto prep = [&]() -> cudaError_t {
            if (l + 1 < L) {
                NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = convTcPrepare<A, Bc, CONV_FWD_RELU>())));
            } else {
                NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = convTcPrepare<A, Bc, CONV_FWD_LINEAR>())));
            }
            if (e == cudaSuccess && l > 0)
                NSDG_CH_SWITCH(CO, A, NSDG_CH_SWITCH(CI, Bc, (e = convTcPrepare<A, Bc, CONV_BWD_DATA>())));
            if (e == cudaSuccess)
                NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = convWeightGradTcPrepare<A, Bc>())));
            return e;
        };
        e = prep();
    }
    if (e == cudaSuccess) {
        // identity normalisation until a dataset sets it
        std::vector<float> st(kWarmNorm, 0.f);
        for (int c = 0; c < kWarmFeat; ++c)
            st[kWarmFeat + c] = 1.f;
        for (int c = 0; c < kWarmTgt; ++c)
            st[2 * kWarmFeat + kWarmTgt + c] = 1.f;
        e = cudaMemcpy(n->stats, st.data(), st.size() * 4, cudaMemcpyHostToDevice);
    }
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
    if (n->dsMem)
        cudaFree(n->dsMem);
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
        if (n->tc && l + 1 < n->L) {
            NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = convTc<A, Bc, CONV_FWD_RELU>(s, B, n->H, n->W, n->act[l],
                                                         w, b, nullptr, n->act[l + 1], nullptr, n->derr))));
        } else if (n->tc) {
            NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = convTc<A, Bc, CONV_FWD_LINEAR>(s, B, n->H, n->W,
                                                         n->act[l], w, b, nullptr, nullptr, n->out, n->derr))));
        } else if (l + 1 < n->L) {
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
    // denominator: sum of the mask times the used channels
    cudaError_t e = cudaSuccess;
    float* invDenom = n->lossPart + (long(n->maxB) * n->H * n->W + 255) / 256 + 1;
    const unsigned lb = static_cast<unsigned>((M + 255) / 256);
    // the weight-gradient partial buffer is free until the first layer's
    // weight gradient: it holds the mask partial sums
    kMaskPartial<<<lb, 256, 0, s>>>(M, n->mask, n->part);
    kInvDenom<<<1, 256, 0, s>>>(static_cast<int>(lb), n->used, n->part, invDenom);
    kLoss<<<lb, 256, 0, s>>>(M, CL, n->used, n->out, n->target, n->mask, invDenom, n->gA, n->lossPart, n->wg);
    kSumPartsBlock<<<1, 256, 0, s>>>(static_cast<int>(lb), 1, n->lossPart, lossDev);
    const int nChunks = static_cast<int>((M + kChunk - 1) / kChunk);
    __nv_bfloat16* gz = n->gA;
    __nv_bfloat16* gnext = n->gB;
    for (int l = n->L - 1; l >= 0 && e == cudaSuccess; --l) {
        const int CI = n->ch[l], CO = n->ch[l + 1];
        const size_t nw = size_t(CO) * 9 * CI;
        // weight gradient: tcgen05 (nine TMEM accumulators of CO columns) or mma.sync
        int nParts = nChunks;
        if (n->tc && 9 * CO <= 512) {
            NSDG_CH_SWITCH(CI, A, NSDG_CH_SWITCH(CO, Bc, (e = convWeightGradTc<A, Bc>(s, B, n->H, n->W, gz, n->act[l],
                                                             n->part, nChunks, n->derr, &nParts))));
        } else {
            dim3 grid(nChunks, 9);
            NSDG_CH_SWITCH(CO, A, NSDG_CH_SWITCH(CI, Bc, (kConvWeightGrad<A, Bc><<<grid, kThreads, 0, s>>>(B, n->H,
                                                              n->W, gz, n->act[l], n->part, n->wg))));
        }
        if (e != cudaSuccess)
            break;
        kSumChunks<<<static_cast<unsigned>((nw + 255) / 256), 256, 0, s>>>(nParts, nw, n->part, n->g32 + n->wOff[l]);
        // bias gradient
        NSDG_CH_SWITCH(CO, A, (kBiasGradPartial<A><<<nChunks, 256, 0, s>>>(M, gz, n->part, n->wg)));
        kSumPartsBlock<<<CO, 256, 0, s>>>(nChunks, CO, n->part, n->g32 + n->bOff[l]);
        // data gradient times relu' of the layer input (not needed for the network input)
        if (l > 0) {
            if (n->tc) {
                NSDG_CH_SWITCH(CO, A, NSDG_CH_SWITCH(CI, Bc, (e = convTc<A, Bc, CONV_BWD_DATA>(s, B, n->H, n->W, gz,
                                                                  n->wt16 + n->wOff[l], nullptr, n->act[l], gnext,
                                                                  nullptr, n->derr))));
            } else {
                NSDG_CH_SWITCH(CO, A, NSDG_CH_SWITCH(CI, Bc, (e = conv<A, Bc, CONV_BWD_DATA>(s, B, n->H, n->W, gz,
                                                                  n->wt16 + n->wOff[l], nullptr, n->act[l], gnext,
                                                                  nullptr))));
            }
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
    kToBf16<<<static_cast<unsigned>((count + 255) / 256), 256, 0, n->stream>>>(count, n->ch[0], n->wg, dev,
        n->act[0]);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Warm start: features, targets, increments, residual
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ size_t ownedNode(int nx, int i, int j, int q)
{
    const int i2 = 2 * i + 1 + (q & 1), j2 = 2 * j + 1 + (q >> 1);
    return size_t(j2) * (2 * nx + 1) + i2;
}

__device__ __forceinline__ void warmFeature(const WarmState& w, size_t e, float* f)
{
    const int i = static_cast<int>(e % w.nx), j = static_cast<int>(e / w.nx);
    f[0] = static_cast<float>(w.hice[e]);
    f[1] = static_cast<float>(w.cice[e]);
    f[2] = w.ice[e] ? 1.f : 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const size_t nd = ownedNode(w.nx, i, j, q);
        const float u = w.u[nd], v = w.v[nd];
        f[3 + q] = u;
        f[7 + q] = v;
        f[33 + q] = u - w.uLast[nd];
        f[37 + q] = v - w.vLast[nd];
    }
    const size_t c = ownedNode(w.nx, i, j, 0);
    f[11] = static_cast<float>(w.ua[c]);
    f[12] = static_cast<float>(w.va[c]);
    f[13] = static_cast<float>(w.uo[c]);
    f[14] = static_cast<float>(w.vo[c]);
#pragma unroll
    for (int k = 0; k < 18; ++k) {
        const float t = w.tdiv[k * w.N + e];
        f[15 + k] = t;
        f[41 + k] = t - w.tdivLast[k * w.N + e];
    }
#pragma unroll
    for (int k = 59; k < kWarmFeat; ++k)
        f[k] = 0.f;
}

__global__ void kWarmFeaturesRaw(WarmState w, float* __restrict__ out)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= w.N)
        return;
    float f[kWarmFeat];
    warmFeature(w, e, f);
#pragma unroll
    for (int k = 0; k < kWarmFeat; ++k)
        out[e * kWarmFeat + k] = f[k];
}

__global__ void kWarmFeaturesNet(WarmState w, const float* __restrict__ stats, __nv_bfloat16* __restrict__ in, int wg)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= w.N)
        return;
    float f[kWarmFeat];
    warmFeature(w, e, f);
#pragma unroll
    for (int k = 0; k < kWarmFeat; ++k)
        in[actChunk(static_cast<long>(e), k >> 3, kWarmFeat, wg) + (k & 7)]
            = __float2bfloat16_rn((f[k] - stats[k]) * stats[kWarmFeat + k]);
}

__device__ __forceinline__ void warmCurrent(const WarmState& w, size_t e, float* t)
{
    const int i = static_cast<int>(e % w.nx), j = static_cast<int>(e / w.nx);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const size_t nd = ownedNode(w.nx, i, j, q);
        t[q] = w.u[nd];
        t[4 + q] = w.v[nd];
    }
#pragma unroll
    for (int k = 0; k < 18; ++k)
        t[8 + k] = w.tdiv[k * w.N + e];
}

__global__ void kWarmBase(WarmState w, float* __restrict__ base, float* __restrict__ mask)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= w.N)
        return;
    mask[e] = w.ice[e] ? 1.f : 0.f;
    float t[kWarmUsed];
    warmCurrent(w, e, t);
#pragma unroll
    for (int k = 0; k < kWarmUsed; ++k)
        base[e * kWarmUsed + k] = t[k];
}

__global__ void kWarmTargets(WarmState w, const float* __restrict__ base, float* __restrict__ out)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= w.N)
        return;
    float t[kWarmUsed];
    warmCurrent(w, e, t);
#pragma unroll
    for (int k = 0; k < kWarmTgt; ++k)
        out[e * kWarmTgt + k] = k < kWarmUsed ? t[k] - base[e * kWarmUsed + k] : 0.f;
}

__global__ void kWarmApply(WarmState w, const float* __restrict__ netOut, const float* __restrict__ stats)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= w.N)
        return;
    const float* tShift = stats + 2 * kWarmFeat;
    const float* tScale = tShift + kWarmTgt;
    const int i = static_cast<int>(e % w.nx), j = static_cast<int>(e / w.nx);
    const float* o = netOut + e * kWarmTgt;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const size_t nd = ownedNode(w.nx, i, j, q);
        if (!w.cg2Dir[nd]) {
            w.u[nd] += o[q] * tScale[q] + tShift[q];
            w.v[nd] += o[4 + q] * tScale[4 + q] + tShift[4 + q];
        }
    }
    if (w.ice[e]) {
#pragma unroll
        for (int k = 0; k < 18; ++k)
            w.tdiv[k * w.N + e] += o[8 + k] * tScale[8 + k] + tShift[8 + k];
    }
}

__global__ void __launch_bounds__(256) kWarmResidualPartial(size_t n, const float* __restrict__ u,
    const float* __restrict__ v, const float* __restrict__ up, const float* __restrict__ vp,
    const float* __restrict__ u0, const float* __restrict__ v0, double* __restrict__ partial)
{
    __shared__ double ws[2][8];
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    double r = 0.0, d = 0.0;
    if (i < n) {
        const double a = double(u[i]) - up[i], b = double(v[i]) - vp[i];
        const double c = double(u[i]) - u0[i], dd = double(v[i]) - v0[i];
        r = a * a + b * b;
        d = c * c + dd * dd;
    }
    for (int off = 16; off > 0; off >>= 1) {
        r += __shfl_down_sync(0xffffffffu, r, off);
        d += __shfl_down_sync(0xffffffffu, d, off);
    }
    if ((threadIdx.x & 31) == 0) {
        ws[0][threadIdx.x >> 5] = r;
        ws[1][threadIdx.x >> 5] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sr = 0.0, sd = 0.0;
        for (int k = 0; k < 8; ++k) {
            sr += ws[0][k];
            sd += ws[1][k];
        }
        partial[2 * blockIdx.x] = sr;
        partial[2 * blockIdx.x + 1] = sd;
    }
}
__global__ void kWarmResidualFinal(size_t nb, const double* __restrict__ partial, double* __restrict__ out)
{
    double sr = 0.0, sd = 0.0;
    for (size_t b = 0; b < nb; ++b) {
        sr += partial[2 * b];
        sd += partial[2 * b + 1];
    }
    out[0] = sr;
    out[1] = sd;
}

// dataset -> network batch (normalised)
__global__ void kGatherBatch(long N, int B, const int* __restrict__ idx, const float* __restrict__ X,
    const float* __restrict__ Y, const float* __restrict__ M, const float* __restrict__ stats,
    __nv_bfloat16* __restrict__ in, float* __restrict__ tgt, float* __restrict__ mask, int wg)
{
    const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
    if (t >= long(B) * N)
        return;
    const int b = static_cast<int>(t / N);
    const long p = t - long(b) * N;
    const long src = long(idx[b]) * N + p;
#pragma unroll 4
    for (int k = 0; k < kWarmFeat; ++k)
        in[actChunk(t, k >> 3, kWarmFeat, wg) + (k & 7)]
            = __float2bfloat16_rn((X[src * kWarmFeat + k] - stats[k]) * stats[kWarmFeat + k]);
    const float* tShift = stats + 2 * kWarmFeat;
    const float* tScale = tShift + kWarmTgt;
#pragma unroll 4
    for (int k = 0; k < kWarmTgt; ++k)
        tgt[t * kWarmTgt + k] = k < kWarmUsed ? (Y[src * kWarmTgt + k] - tShift[k]) / tScale[k] : 0.f;
    mask[t] = M[src];
}

// per-channel sums and sums of squares over `rows` rows of `C` channels (masked
// rows only), one partial per block
__global__ void kChannelMoments(long rows, int C, const float* __restrict__ a, const float* __restrict__ maskRows,
    double* __restrict__ partial)
{
    const int c = blockIdx.y;
    double s = 0.0, s2 = 0.0;
    for (long r = blockIdx.x * long(blockDim.x) + threadIdx.x; r < rows; r += long(gridDim.x) * blockDim.x) {
        if (maskRows[r] == 0.f)
            continue;
        const double v = a[r * C + c];
        s += v;
        s2 += v * v;
    }
    __shared__ double ws[2][8];
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        s2 += __shfl_down_sync(0xffffffffu, s2, off);
    }
    if ((threadIdx.x & 31) == 0) {
        ws[0][threadIdx.x >> 5] = s;
        ws[1][threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a0 = 0, a1 = 0;
        for (int k = 0; k < 8; ++k) {
            a0 += ws[0][k];
            a1 += ws[1][k];
        }
        partial[(long(c) * gridDim.x + blockIdx.x) * 2] = a0;
        partial[(long(c) * gridDim.x + blockIdx.x) * 2 + 1] = a1;
    }
}

__global__ void kWarmDecide(cudaGraphConditionalHandle h, const double* __restrict__ res, double kappa,
    WarmRecord rec)
{
    const double r = res[0], d = res[1];
    const double ratio = d > 0.0 ? sqrt(r / d) : (r > 0.0 ? INFINITY : 0.0);
    const bool ok = *rec.enabled != 0 && *rec.warmErr == 0 && isfinite(r) && isfinite(d) && ratio <= kappa;
    *rec.lastRatio = ratio;
    rec.counts[ok ? 0 : 1] += 1;
    *rec.warmErr = 0;
    cudaGraphSetConditional(h, ok ? 0u : 1u);
}

__global__ void kWarmAudit(const double* __restrict__ res, double tol, WarmRecord rec)
{
    const double r = res[0], d = res[1];
    const double err = d > 0.0 ? sqrt(r / d) : (r > 0.0 ? INFINITY : 0.0);
    const bool ok = *rec.warmErr == 0 && isfinite(r) && isfinite(d) && err <= tol;
    *rec.lastError = err;
    *rec.enabled = ok ? 1 : 0;
    rec.counts[2] += 1;
    if (!ok)
        rec.counts[3] += 1;
    *rec.warmErr = 0;
}

__global__ void kWarmSave(size_t n, const float* __restrict__ src, float* __restrict__ d1, float* __restrict__ d2)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i < n) {
        const float x = src[i];
        d1[i] = x;
        if (d2)
            d2[i] = x;
    }
}

__global__ void kNarrow(size_t n, const double* __restrict__ src, float* __restrict__ dst)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i < n)
        dst[i] = static_cast<float>(src[i]);
}

__global__ void kCopyF32(size_t n, const float* __restrict__ src, float* __restrict__ dst)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i < n)
        dst[i] = src[i];
}

unsigned gridOf(size_t n) { return static_cast<unsigned>((n + 255) / 256); }

} // namespace

cudaError_t launchWarmDecide(cudaStream_t s, cudaGraphConditionalHandle h, const double* res, double kappa,
    const WarmRecord& rec)
{
    kWarmDecide<<<1, 1, 0, s>>>(h, res, kappa, rec);
    return cudaGetLastError();
}
cudaError_t launchWarmAudit(cudaStream_t s, const double* res, double tol, const WarmRecord& rec)
{
    kWarmAudit<<<1, 1, 0, s>>>(res, tol, rec);
    return cudaGetLastError();
}
cudaError_t launchWarmSave(cudaStream_t s, size_t n, const float* src, float* dst1, float* dst2)
{
    kWarmSave<<<gridOf(n), 256, 0, s>>>(n, src, dst1, dst2);
    return cudaGetLastError();
}
cudaError_t launchNarrow(cudaStream_t s, size_t n, const double* src, float* dst)
{
    kNarrow<<<gridOf(n), 256, 0, s>>>(n, src, dst);
    return cudaGetLastError();
}

cudaError_t launchCopyF32(cudaStream_t s, size_t n, const float* src, float* dst)
{
    kCopyF32<<<gridOf(n), 256, 0, s>>>(n, src, dst);
    return cudaGetLastError();
}

cudaError_t launchWarmFeaturesRaw(cudaStream_t s, const WarmState& w, float* out)
{
    kWarmFeaturesRaw<<<gridOf(w.N), 256, 0, s>>>(w, out);
    return cudaGetLastError();
}
cudaError_t launchWarmFeaturesNet(cudaStream_t s, const WarmState& w, NetImpl* net)
{
    kWarmFeaturesNet<<<gridOf(w.N), 256, 0, s>>>(w, net->stats, net->act[0], net->wg);
    return cudaGetLastError();
}
cudaError_t launchWarmBase(cudaStream_t s, const WarmState& w, float* base, float* mask)
{
    kWarmBase<<<gridOf(w.N), 256, 0, s>>>(w, base, mask);
    return cudaGetLastError();
}
cudaError_t launchWarmTargets(cudaStream_t s, const WarmState& w, const float* base, float* out)
{
    kWarmTargets<<<gridOf(w.N), 256, 0, s>>>(w, base, out);
    return cudaGetLastError();
}
cudaError_t launchWarmApply(cudaStream_t s, const WarmState& w, NetImpl* net)
{
    kWarmApply<<<gridOf(w.N), 256, 0, s>>>(w, net->out, net->stats);
    return cudaGetLastError();
}
size_t warmResidualPartials(size_t n) { return 2 * gridOf(n); }
cudaError_t launchWarmResidual(cudaStream_t s, size_t n, const float* u, const float* v, const float* uPrev,
    const float* vPrev, const float* u0, const float* v0, double* partial, double* out)
{
    kWarmResidualPartial<<<gridOf(n), 256, 0, s>>>(n, u, v, uPrev, vPrev, u0, v0, partial);
    kWarmResidualFinal<<<1, 1, 0, s>>>(gridOf(n), partial, out);
    return cudaGetLastError();
}

bool netIsWarmShaped(NetImpl* n, int nx, int ny)
{
    return n && n->W == nx && n->H == ny && n->ch[0] == kWarmFeat && n->ch[n->L] == kWarmTgt
        && n->used == kWarmUsed;
}

int netDatasetReserve(NetImpl* n, int capacity, std::string& err)
{
    if (capacity < 1) {
        err = "dataset capacity must be positive";
        return NSDG_ERR_BAD_ARG;
    }
    if (n->ch[0] != kWarmFeat || n->ch[n->L] != kWarmTgt) {
        err = "the dataset needs a network with the warm-start input and output channel counts";
        return NSDG_ERR_BAD_ARG;
    }
    const size_t N = size_t(n->H) * n->W;
    const size_t bytes = a256(size_t(capacity) * N * kWarmFeat * 4) + a256(size_t(capacity) * N * kWarmTgt * 4)
        + a256(size_t(capacity) * N * 4) + a256(size_t(2) * 80 * 1024 * 8);
    if (n->dsMem)
        cudaFree(n->dsMem);
    n->dsMem = nullptr;
    if (cudaMalloc(&n->dsMem, bytes) != cudaSuccess) {
        cudaGetLastError();
        err = "dataset: device allocation failed";
        return NSDG_ERR_CUDA;
    }
    char* p = static_cast<char*>(n->dsMem);
    n->dsX = reinterpret_cast<float*>(p);
    p += a256(size_t(capacity) * N * kWarmFeat * 4);
    n->dsY = reinterpret_cast<float*>(p);
    p += a256(size_t(capacity) * N * kWarmTgt * 4);
    n->dsM = reinterpret_cast<float*>(p);
    p += a256(size_t(capacity) * N * 4);
    n->dPart = reinterpret_cast<double*>(p);
    n->dsCap = capacity;
    return NSDG_OK;
}
float* netDatasetFeatures(NetImpl* n, int slot) { return n->dsX + size_t(slot) * n->H * n->W * kWarmFeat; }
float* netDatasetTargets(NetImpl* n, int slot) { return n->dsY + size_t(slot) * n->H * n->W * kWarmTgt; }
float* netDatasetMask(NetImpl* n, int slot) { return n->dsM + size_t(slot) * n->H * n->W; }
int netDatasetCapacity(NetImpl* n) { return n->dsCap; }

int netDatasetNormalise(NetImpl* n, int count, std::string& err)
{
    if (count < 1 || count > n->dsCap) {
        err = "normalise: bad sample count";
        return NSDG_ERR_BAD_ARG;
    }
    const long rows = long(count) * n->H * n->W;
    const int blocks = 80;
    std::vector<float> st(2 * kWarmFeat + 2 * kWarmTgt, 0.f);
    // number of sea cells: the mask's own masked sum
    double msum = 0;
    {
        kChannelMoments<<<dim3(blocks, 1), 256, 0, n->stream>>>(rows, 1, n->dsM, n->dsM, n->dPart);
        std::vector<double> part(size_t(2) * blocks);
        cudaError_t e = cudaMemcpyAsync(part.data(), n->dPart, part.size() * 8, cudaMemcpyDeviceToHost, n->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(n->stream);
        if (e != cudaSuccess) {
            err = std::string("normalise: ") + cudaGetErrorString(e);
            return NSDG_ERR_CUDA;
        }
        for (int b = 0; b < blocks; ++b)
            msum += part[2 * b];
    }
    for (int pass = 0; pass < 2; ++pass) {
        const int C = pass == 0 ? kWarmFeat : kWarmTgt;
        const float* a = pass == 0 ? n->dsX : n->dsY;
        kChannelMoments<<<dim3(blocks, C), 256, 0, n->stream>>>(rows, C, a, n->dsM, n->dPart);
        std::vector<double> part(size_t(2) * blocks * C);
        cudaError_t e = cudaMemcpyAsync(part.data(), n->dPart, part.size() * 8, cudaMemcpyDeviceToHost, n->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(n->stream);
        if (e != cudaSuccess) {
            err = std::string("normalise: ") + cudaGetErrorString(e);
            return NSDG_ERR_CUDA;
        }
        for (int c = 0; c < C; ++c) {
            double s = 0, s2 = 0;
            for (int b = 0; b < blocks; ++b) {
                s += part[(size_t(c) * blocks + b) * 2];
                s2 += part[(size_t(c) * blocks + b) * 2 + 1];
            }
            const double mean = msum > 0 ? s / msum : 0.0;
            const double var = msum > 0 ? std::max(s2 / msum - mean * mean, 0.0) : 0.0;
            const double sd = std::sqrt(var);
            if (pass == 0) {
                st[c] = static_cast<float>(mean);
                st[kWarmFeat + c] = sd > 1e-30 ? static_cast<float>(1.0 / sd) : 0.f;
            } else {
                st[2 * kWarmFeat + c] = static_cast<float>(mean);
                st[2 * kWarmFeat + kWarmTgt + c] = sd > 1e-30 ? static_cast<float>(sd) : 1.f;
            }
        }
    }
    if (cudaMemcpy(n->stats, st.data(), st.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        err = "normalise: upload failed";
        return NSDG_ERR_CUDA;
    }
    return NSDG_OK;
}

int netTrain(NetImpl* n, int count, int iterations, int batch, float lr, unsigned long long seed, float* loss,
    std::string& err)
{
    if (count < 1 || count > n->dsCap || batch < 1 || batch > n->maxB || iterations < 1) {
        err = "train: bad arguments";
        return NSDG_ERR_BAD_ARG;
    }
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int> pick(0, count - 1);
    const long N = long(n->H) * n->W;
    std::vector<int> idx(batch);
    float* lossDev = n->lossPart + (N * n->maxB + 255) / 256; // one spare float after the loss partials
    std::vector<float> last;
    for (int it = 0; it < iterations; ++it) {
        for (int& i : idx)
            i = pick(rng);
        cudaError_t e = cudaMemcpyAsync(n->dIdx, idx.data(), batch * 4, cudaMemcpyHostToDevice, n->stream);
        if (e == cudaSuccess) {
            const long T = long(batch) * N;
            kGatherBatch<<<static_cast<unsigned>((T + 255) / 256), 256, 0, n->stream>>>(N, batch, n->dIdx, n->dsX,
                n->dsY, n->dsM, n->stats, n->act[0], n->target, n->mask, n->wg);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = netForward(n, n->stream, batch);
        if (e == cudaSuccess) e = netLossBackward(n, batch, lossDev);
        if (e == cudaSuccess) e = netAdam(n, lr, 0.9f, 0.999f, 1e-8f);
        float l = 0.f;
        if (e == cudaSuccess && it + 20 >= iterations) {
            e = cudaMemcpyAsync(&l, lossDev, 4, cudaMemcpyDeviceToHost, n->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(n->stream);
            last.push_back(l);
        }
        if (e != cudaSuccess) {
            err = std::string("train: ") + cudaGetErrorString(e);
            return NSDG_ERR_CUDA;
        }
    }
    double s = 0;
    for (float v : last)
        s += v;
    if (loss)
        *loss = static_cast<float>(s / std::max<size_t>(1, last.size()));
    return NSDG_OK;
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

nsdg::NetImpl* nsdg::netImplOf(nsdg_net* h) { return h ? h->impl : nullptr; }

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

// After the stream has been synchronised: the tensor-core convolutions'
// error word (a bounded wait ran out), reported once and cleared.
static int netDeviceStatus(nsdg_net* h)
{
    int word = 0;
    cudaError_t e = cudaMemcpy(&word, h->impl->derr, sizeof word, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && word != 0) {
        cudaMemset(h->impl->derr, 0, sizeof word);
        h->err = "a bounded wait of a tensor-core convolution ran out";
        return NSDG_ERR_CUDA;
    }
    if (e != cudaSuccess) {
        h->err = cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
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
    return netDeviceStatus(h);
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

int nsdg_net_time_forward(nsdg_net* h, int batch, int reps, float* ms)
{
    if (!h || batch < 1 || batch > h->impl->maxB || reps < 1 || !ms)
        return NSDG_ERR_BAD_ARG;
    NetImpl* n = h->impl;
    cudaStream_t s = netStream(n);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    if (e == cudaSuccess)
        e = cudaEventRecord(e0, s);
    for (int r = 0; r < reps && e == cudaSuccess; ++r)
        e = netForward(n, s, batch);
    if (e == cudaSuccess)
        e = cudaEventRecord(e1, s);
    if (e == cudaSuccess)
        e = cudaEventSynchronize(e1);
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(ms, e0, e1);
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        h->err = cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
    *ms /= float(reps);
    return netDeviceStatus(h);
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

int nsdg_net_get_normalisation(nsdg_net* h, float* host, size_t n)
{
    if (!h || !host)
        return NSDG_ERR_BAD_ARG;
    if (n != NSDG_NET_NORM_FLOATS) {
        h->err = "normalisation: expected NSDG_NET_NORM_FLOATS floats";
        return NSDG_ERR_SIZE_MISMATCH;
    }
    const cudaError_t e = cudaMemcpy(host, h->impl->stats, n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        h->err = std::string("normalisation: ") + cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
    return NSDG_OK;
}

int nsdg_net_set_normalisation(nsdg_net* h, const float* host, size_t n)
{
    if (!h || !host)
        return NSDG_ERR_BAD_ARG;
    if (n != NSDG_NET_NORM_FLOATS) {
        h->err = "normalisation: expected NSDG_NET_NORM_FLOATS floats";
        return NSDG_ERR_SIZE_MISMATCH;
    }
    cudaError_t e = cudaStreamSynchronize(h->impl->stream);
    if (e == cudaSuccess) e = cudaMemcpy(h->impl->stats, host, n * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        h->err = std::string("normalisation: ") + cudaGetErrorString(e);
        return NSDG_ERR_CUDA;
    }
    return NSDG_OK;
}

int nsdg_net_dataset_reserve(nsdg_net* h, int capacity)
{
    if (!h)
        return NSDG_ERR_BAD_ARG;
    return netDatasetReserve(h->impl, capacity, h->err);
}

int nsdg_net_dataset_normalise(nsdg_net* h, int count)
{
    if (!h)
        return NSDG_ERR_BAD_ARG;
    return netDatasetNormalise(h->impl, count, h->err);
}

int nsdg_net_train(nsdg_net* h, int count, int iterations, int batch, float lr, unsigned long long seed, float* loss)
{
    if (!h)
        return NSDG_ERR_BAD_ARG;
    return netTrain(h->impl, count, iterations, batch, lr, seed, loss, h->err);
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
