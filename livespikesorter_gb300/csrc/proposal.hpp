// proposal.hpp -- sorter-side interface of the learned proposal gate (kernels in proposal.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lss {

struct PropGate;

// Device copy of one gate: BF16 weights, FP32 biases, the template -> neighbourhood table of
// wall3 [T][K][C] (host).  Throws LoadError / CudaError.
PropGate* prop_gate_create(int device, const float* params, float logit_threshold, int dilate, const float* wall3,
                           int T, int K, int C);
void prop_gate_destroy(PropGate* g);

// Enqueue the gate of nb windows on st: the network over the whitened windows Z [nb][W][C], then
// Bt [nb][W][T] := -1e30 at the interior samples whose (owner(t), window) cell is closed.  Grows
// the gate's buffers first when W or nb exceed them (synchronizing st).  Returns the launches.
int prop_gate_run(PropGate* g, const float* Z, float* Bt, int nb, int W, int nt, cudaStream_t st);

// Cells evaluated and left open since the gate was created (synchronizes st).
void prop_gate_stats(PropGate* g, cudaStream_t st, int64_t* cells, int64_t* open);

}  // namespace lss
