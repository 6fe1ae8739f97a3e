// mlp_internal.h -- what the batch solver needs from the warm-start network.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "gbpf.h"

namespace gbpf {

// Feature and output layout of a warm-start network (see gbpf_mlp_create):
// inputs [Pliq of every bus | Qliq of every bus | V0 of every bus] padded with
// zeros to kin (a multiple of 8), outputs [|V| of every bus | theta of every bus].
struct MlpShape {
    int n_in, kin, n_out, outp, device;  // outp: n_out rounded up to a multiple of 8 (row length of out)
    const float *in_mean, *in_iscale;    // device [n_in]: x_norm = (x - mean) * iscale
    const float *out_mean, *out_scale;   // device [n_out]: y = y_norm * scale + mean
    const float *h_out_mean;             // host copy of out_mean
};
MlpShape mlp_shape(const gbpf_mlp *m);

// Inference workspace owned by a caller, so that callers that share a
// network (two batches in flight) can run its forward pass at the same time
// on their own streams.  Grows to the largest n seen; remade for another
// network.
struct MlpWork;
MlpWork *mlp_work_create();
void mlp_work_free(MlpWork *w);

// Forward pass of normalised bf16 features X [n, kin] (device) into normalised
// outputs out [n, outp] (device, fp32), on stream st, in workspace w (null:
// the network's own).
gbpf_status mlp_infer(gbpf_mlp *m, const __nv_bfloat16 *X, int n, float *out, cudaStream_t st,
                      MlpWork *w = nullptr);

}  // namespace gbpf
