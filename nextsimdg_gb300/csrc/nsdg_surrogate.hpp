// nsdg_surrogate.hpp — host-side interface of the warm-start network
// (nsdg_surrogate.cu): creation, the forward and backward passes, Adam, and
// raw access to the device buffers for the feature/increment kernels.
#pragma once

#include <cstddef>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <string>

namespace nsdg {

struct NetImpl;

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

} // namespace nsdg
