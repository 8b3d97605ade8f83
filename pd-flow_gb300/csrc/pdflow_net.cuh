// Internal interface between the solver and the warm-start network
// (pdflow_net.cu); the public C ABI is include/pdflow_net.h.
#pragma once
#include <cuda_runtime.h>

#include "pdflow_kernels.cuh"

struct pdflow_net;

namespace pdflow {

// Gathers both frames' 60x80 level planes of nb pairs (mapped slots) into the
// network's input buffer, on stream st.
int net_gather_input(pdflow_net* n, const PyrLevel& old_l, const PyrLevel& new_l, size_t pstride,
                     const unsigned* map, int nb, cudaStream_t st);
float* net_input_buffer(pdflow_net* n);
// The same gather into a caller buffer out [nb][4][4800].
cudaError_t launch_gather_seed_input(const PyrLevel& old_l, const PyrLevel& new_l, size_t pstride,
                                     const unsigned* map, int nb, float* out, cudaStream_t st);
// Forward pass on inputs [nb][4][4800] -> seed [nb][3][4800] (du, dv, dw), on
// the network's stream.
int net_seed(pdflow_net* n, int nb, const float* input, float* seed);
unsigned net_max_batch(const pdflow_net* n);
// Unique per network created in this process (never reused, unlike addresses).
unsigned long long net_uid(const pdflow_net* n);
// Kernel launches of net_seed for nb inputs.
unsigned net_seed_launches(const pdflow_net* n, int nb);
cudaStream_t net_stream(const pdflow_net* n);
void net_set_stream_internal(pdflow_net* n, cudaStream_t st);

}  // namespace pdflow
