// Internal interface of the learned preconditioner (unet.cu) for the flexible CG solver.
#pragma once

#include <cuda_runtime.h>

#include "lentils_gb300.h"

namespace lentils {

// z = u + s * net(u / s, feat), u = dinv * r, s = rms(u); one H x W sample; no synchronisation
int unet_precondition(lentils_unet *net, const float *r, const float *dinv, const float *feat,
                      float *z, cudaStream_t s);
// one-time set-up of the forward kernels (call before capturing unet_precondition in a graph)
int unet_prepare(lentils_unet *net);
// H * W of the network's grid
int unet_size(const lentils_unet *net);
// reads the tensor-core wait flag (synchronous)
int unet_error_flag_device(lentils_unet *net, int *flag);

}  // namespace lentils
