// learned.cuh -- the gauge-covariant network used as a preconditioner.
//
// Four linear layers alternate the sub-lattice: even -> odd -> even -> odd ->
// even.  A layer reads C = 8 input channels (each a colour vector per site)
// on one parity and writes C channels on the other:
//   h_{d,c}(x) = s U_mu(x) in_c(x+mu)            d = mu     (forward hop)
//   h_{d,c}(x) = s U_mu(x-mu)^+ in_c(x-mu)       d = 4+mu   (backward hop)
//   out_n(x)   = sum_{d,c} W[d*C + c][n] h_{d,c}(x)
// with s the staggered sign of the link.  Real weights commute with the
// SU(3) action, so the layer is gauge covariant.  The channel mixing is a
// dense contraction [sites x 64] x [64 x 8] per colour component, done with
// tcgen05 BF16 MMA (FP32 accumulation in tensor memory).
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "common.cuh"

namespace ost {

static constexpr int NET_C = 8;          // channels per colour
static constexpr int NET_K = 8 * NET_C;  // hops x channels
static constexpr int NET_N = 16;         // MMA N (output channels padded to 16)
static constexpr int NET_LAYERS = 4;

struct NetBuffers {
  // activations: [layer][C][3][sizeh] bf16x2 (complex); layer l is the input of layer l
  __nv_bfloat162* act;
  float* grad_a;        // [C][3][sizeh] float2 gradient, two ping-pong buffers
  float* grad_b;
  float* w_master;      // [L][64][8] FP32 master weights
  float* adam_m;        // [L][64][8]
  float* adam_v;
  float* dw;            // [L][64][8]
  float* dw_partials;   // [grid][64][8]
  __nv_bfloat16* w_mma; // [L][16][64] BF16, K-major operand layout source
  int* err;             // bounded-wait failures
  double* loss;         // [2]
};

// layer l of the forward pass: act[l] (parity 1-P_OUT) -> act[l+1] or, for the
// last layer, channel 0 into out_f32 (float2 vec3 on parity P_OUT)
void net_layer_forward(const NetBuffers& nb, int layer, const float2* u32, const unsigned char* signs,
                       float2* out_f32, cudaStream_t st);
// input of layer 0 from a float2 vec3 field (channel 0; channels 1..7 zero)
void net_load_input(const NetBuffers& nb, const float2* r, cudaStream_t st);
// residual loss of a batch entry from w = A (z - x) and aw = A w:
// loss (+)= scale |w|^2, grad_a channel 0 = 2 scale aw, channels 1..7 zero
void net_residual_loss_grad(const NetBuffers& nb, const float2* w, const float2* aw, double scale, int accumulate,
                            cudaStream_t st);
// backward of layer l: grad (output side) -> dW[l] (+=) and grad (input side)
void net_layer_backward(const NetBuffers& nb, int layer, const float2* u32, const unsigned char* signs,
                        const float* g_out, float* g_in, int need_g_in, cudaStream_t st);
void net_adam_step(const NetBuffers& nb, float lr, float beta1, float beta2, float eps, int t, cudaStream_t st);
void net_sync_weights(const NetBuffers& nb, cudaStream_t st);   // master FP32 -> BF16 MMA copy
void net_zero_dw(const NetBuffers& nb, cudaStream_t st);
// bounded mbarrier wait with (signal = 1) or without its arrival; a timeout
// sets nb.err like a lost MMA completion
void net_wait_selftest(const NetBuffers& nb, int signal, long polls, cudaStream_t st);

}  // namespace ost
