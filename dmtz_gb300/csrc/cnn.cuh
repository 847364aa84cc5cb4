// cnn.cuh — what the correction library and the learned-proposal network
// share: the per-vertex feature layout and the network's internal entry
// points (no counterpart in the reference).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/dmtz.h"

namespace dmtz_cnn_impl {

// Features, bf16, channels-last [vertex][16]:
//   0      (g - f) / bound                        in [-1, 1]
//   1      1 where the vertex's own cells differ in criticality between the
//          gradients of f and g, else 0
//   2..15  tanh((f(u) - f(v)) / (4 bound)) for the 14 Freudenthal neighbours
//          u of v in stencil order, 0 outside the grid
constexpr int kFeat = 16;

// Forward pass on `stream`: feat (device, V x 16 bf16) -> out (device, V
// floats, the pre-tanh proposal).  train != 0 keeps every activation for a
// following backward pass.  Synchronous only if the caller synchronises.
dmtz_status forward_on(dmtz_cnn *net, int W, int H, int D, const __nv_bfloat16 *feat, float *out, int train,
                       cudaStream_t stream);

// net-owned device scratch for the features / mask / output of a warm start
dmtz_status scratch(dmtz_cnn *net, int64_t V, __nv_bfloat16 **feat, uint8_t **active, float **out);

const std::string &error_of(const dmtz_cnn *net);
int device_of(const dmtz_cnn *net);
float min_drop_of(const dmtz_cnn *net);

}  // namespace dmtz_cnn_impl
