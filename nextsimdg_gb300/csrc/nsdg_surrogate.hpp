// nsdg_surrogate.hpp — host-side interface of the warm-start network
// (nsdg_surrogate.cu): creation, the forward and backward passes, Adam, and
// raw access to the device buffers for the feature/increment kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <string>

struct nsdg_net;

namespace nsdg {

struct NetImpl;
NetImpl* netImplOf(nsdg_net* h);

// channels: L+1 counts (16, 32 or 48); `used` output channels enter the loss.
int netCreate(int L, const int* channels, int H, int W, int maxBatch, int used, unsigned long long seed,
    NetImpl** out, std::string& err);
void netDestroy(NetImpl* n);
cudaError_t netRefresh(NetImpl* n);
cudaError_t netForward(NetImpl* n, cudaStream_t s, int batch);
cudaError_t netLossBackward(NetImpl* n, int batch, float* lossDev);
cudaError_t netAdam(NetImpl* n, float lr, float b1, float b2, float eps);
cudaError_t netInputFromFloat(NetImpl* n, long count, const float* dev);

cudaStream_t netStream(NetImpl* n);
__nv_bfloat16* netInput(NetImpl* n);   // [B][H][W][ch0]
float* netOutput(NetImpl* n);          // [B][H][W][chL]
float* netTarget(NetImpl* n);          // [B][H][W][chL]
float* netMask(NetImpl* n);            // [B][H][W]
int netChannels(NetImpl* n, int l);
int netLayers(NetImpl* n);
size_t netParamCount(NetImpl* n);
float* netParams(NetImpl* n);
float* netGrads(NetImpl* n);

// ---- warm start of the mEVP sub-cycle --------------------------------------
// Feature and target layouts per cell (i, j) of the dynamics grid, the
// "owned" CG2 nodes of the cell being q = 0: (2i+1, 2j+1), 1: (2i+2, 2j+1),
// 2: (2i+1, 2j+2), 3: (2i+2, 2j+2) (every node but the domain's left column
// and bottom row belongs to exactly one cell):
//   features (kWarmFeat = 64): [0] h, [1] A, [2] sea mask, [3..6] u at q0..q3,
//     [7..10] v at q0..q3, [11..14] wind and ocean velocity at the cell centre,
//     [15..32] the 18 divergence coefficients, [33..40] u, v minus their values
//     at the start of the previous sub-cycle, [41..58] the same for the
//     divergence coefficients, zero padding;
//   targets (kWarmTgt = 32, kWarmUsed = 26 used): increments of u at q0..q3,
//     v at q0..q3 and of the 18 divergence coefficients, zero padding.
constexpr int kWarmFeat = 64;
constexpr int kWarmTgt = 32;
constexpr int kWarmUsed = 26;
constexpr int kWarmNorm = 2 * kWarmFeat + 2 * kWarmTgt; // feature mean, 1/std; target mean, std

struct WarmState {
    int nx, ny;
    size_t N;
    const double* hice; // component 0 = cell average
    const double* cice;
    const uint8_t* ice;
    const uint8_t* cg2Dir;
    float* u;           // FP32 iterate (CG2)
    float* v;
    const double* ua;
    const double* va;
    const double* uo;
    const double* vo;
    float* tdiv;        // [18][N]
    const float* uLast; // u, v, tdiv at the start of the previous sub-cycle
    const float* vLast;
    const float* tdivLast;
};
// raw FP32 features [N][kWarmFeat]
cudaError_t launchWarmFeaturesRaw(cudaStream_t s, const WarmState& w, float* out);
// normalised BF16 features into the network input (batch slot 0)
cudaError_t launchWarmFeaturesNet(cudaStream_t s, const WarmState& w, NetImpl* net);
// base values [N][kWarmUsed] (u, v at the owned nodes, tdiv) and raw targets
// [N][kWarmTgt] = current - base
// and the loss mask [N] (1 on sea cells)
cudaError_t launchWarmBase(cudaStream_t s, const WarmState& w, float* base, float* mask);
cudaError_t launchWarmTargets(cudaStream_t s, const WarmState& w, const float* base, float* out);
// u, v, tdiv += de-normalised network output (Dirichlet nodes and land cells untouched)
cudaError_t launchWarmApply(cudaStream_t s, const WarmState& w, NetImpl* net);
// sums over CG2 nodes: out[0] = |(u,v) - (uPrev,vPrev)|^2, out[1] = |(u,v) - (u0,v0)|^2
cudaError_t launchWarmResidual(cudaStream_t s, size_t n, const float* u, const float* v, const float* uPrev,
    const float* vPrev, const float* u0, const float* v0, double* partial, double* out);
size_t warmResidualPartials(size_t n);

// dataset of training samples held on the device next to the network
int netDatasetReserve(NetImpl* n, int capacity, std::string& err);
float* netDatasetFeatures(NetImpl* n, int slot); // raw [N][kWarmFeat]
float* netDatasetTargets(NetImpl* n, int slot);  // raw [N][kWarmTgt]
float* netDatasetMask(NetImpl* n, int slot);     // [N]
int netDatasetCapacity(NetImpl* n);
// per-channel mean / std of the first `count` samples (features and targets)
int netDatasetNormalise(NetImpl* n, int count, std::string& err);
// Adam on random batches of the first `count` samples; *loss = mean of the last 20 losses
int netTrain(NetImpl* n, int count, int iterations, int batch, float lr, unsigned long long seed, float* loss,
    std::string& err);
bool netIsWarmShaped(NetImpl* n, int nx, int ny);
// Device-side record of the warm start (counts: accepted, fallbacks, audited,
// audited-and-rejected sub-cycles).
struct WarmRecord {
    long long* counts;  // [4]
    int* warmErr;       // numeric fault of the warm attempt (private to it)
    int* enabled;       // 1 while the last audit allows warm sub-cycles
    double* lastRatio;
    double* lastError;
};
// Acceptance test of a warm sub-cycle, launched inside the update graph:
// ratio = sqrt(res[0] / res[1]); accepted when the warm start is enabled, the
// warm iterations raised no device error and ratio <= kappa.  Sets the graph
// conditional `h` to 1 for a fallback, counts, stores the ratio and clears
// the warm error word.
cudaError_t launchWarmDecide(cudaStream_t s, cudaGraphConditionalHandle h, const double* res, double kappa,
    const WarmRecord& rec);
// Audit against the plain sub-cycle: err = sqrt(res[0] / res[1]) with
// res from launchWarmResidual(plain result, warm result, start); enables the
// warm start when the warm attempt raised no device error and err <= tol.
cudaError_t launchWarmAudit(cudaStream_t s, const double* res, double tol, const WarmRecord& rec);
// dst1 = dst2 = src (dst2 may be null)
cudaError_t launchWarmSave(cudaStream_t s, size_t n, const float* src, float* dst1, float* dst2);
// dst = (float) src
cudaError_t launchNarrow(cudaStream_t s, size_t n, const double* src, float* dst);
// float copy kernel (usable inside conditional graph bodies)
cudaError_t launchCopyF32(cudaStream_t s, size_t n, const float* src, float* dst);

} // namespace nsdg
