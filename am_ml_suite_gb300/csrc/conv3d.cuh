// conv3d.cuh -- BF16 3x3x3 convolutions (FP32 accumulate) on tensor cores for the
// learned preconditioner, plus the small tensor kernels around them.
//
// Tensors are channels-last: t[((n*Dz + z)*Dy + y)*Dx + x][c] with a channel
// stride (>= the channels used) and a channel offset, so a convolution can read
// or write one slice of a concatenation buffer in place.  Channel counts are
// multiples of 16.  Weights are w[tap][cout][cin] (cin contiguous), tap =
// (dz*3 + dy)*3 + dx; every convolution is stride 1 with zero padding 1.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace amk {

struct TensorView {
    void *p;       // __nv_bfloat16 or float
    int cstride;   // elements between consecutive voxels
    int coff;      // first channel of the slice
};

struct Grid5 {
    int n, dz, dy, dx;
    long long voxels() const { return (long long)n * dz * dy * dx; }
};

// Which kernels the convolutions run on: 1 (the default) tcgen05.mma with TMEM
// accumulators and tensor-copy staging (conv3d_tc.cu); 0 the legacy
// mma.sync/ldmatrix/cp.async kernels (conv3d.cu), kept as the baseline the
// tensor-core kernels are measured and checked against.
void conv3d_set_impl(int impl);
int conv3d_impl();
// Error flag of the tensor-core kernels' bounded waits (1 = a wait ran out), read
// after the work queued on `st`; clear resets it.
cudaError_t conv3d_tc_error(int *flag, bool clear, cudaStream_t st);
cudaError_t conv3d_fwd_tc(const Grid5 &g, TensorView x, int cin, const __nv_bfloat16 *w, int cout, TensorView y,
                          TensorView yf, int relu, cudaStream_t st);
cudaError_t conv3d_wgrad_tc(const Grid5 &g, TensorView x, int cin, TensorView dy, int cout, float *dw,
                            cudaStream_t st);

// y = conv(x, w); relu; output BF16 (y) and/or FP32 (yf).  Cin, Cout multiples
// of 16.
cudaError_t conv3d_fwd(const Grid5 &g, TensorView x, int cin, const __nv_bfloat16 *w, int cout, TensorView y,
                       TensorView yf, int relu, cudaStream_t st);
// dw[tap][cout][cin] += sum_v dy[v][cout] x[v + tap][cin]   (FP32 atomics)
cudaError_t conv3d_wgrad(const Grid5 &g, TensorView x, int cin, TensorView dy, int cout, float *dw, cudaStream_t st);
// wt[tap][cin][cout] = w[26 - tap][cout][cin]: the weights of the backward-data
// convolution (dx = conv(dy, wt))
cudaError_t conv3d_flip_transpose(const __nv_bfloat16 *w, int cout, int cin, __nv_bfloat16 *wt, cudaStream_t st);
// g = g * (y > 0) on `c` channels (ReLU backward; y the post-activation output)
cudaError_t relu_bwd(const Grid5 &g, TensorView grad, TensorView y, int c, cudaStream_t st);
// 2x2x2 mean pool (dims of the output grid g; input grid 2x in z, y, x)
cudaError_t avgpool2_fwd(const Grid5 &g, TensorView in, TensorView out, int c, cudaStream_t st);
// din (+)= dout / 8 broadcast (accumulate != 0 adds to din)
cudaError_t avgpool2_bwd(const Grid5 &g, TensorView dout, TensorView din, int c, int accumulate, cudaStream_t st);
// nearest 2x upsampling (g: the fine output grid; input grid half of it)
cudaError_t upsample2_fwd(const Grid5 &g, TensorView in, TensorView out, int c, cudaStream_t st);
// din = sum of the 8 fine gradients (g: the fine grid)
cudaError_t upsample2_bwd(const Grid5 &g, TensorView dout, TensorView din, int c, cudaStream_t st);
// Adam on FP32 master weights; writes the BF16 copy.  t: step (1-based)
cudaError_t adam_step(float *w, float *m, float *v, const float *grad, __nv_bfloat16 *wb, long long n, float lr,
                      float beta1, float beta2, float eps, int t, float grad_scale, cudaStream_t st);
cudaError_t f32_to_bf16(const float *a, __nv_bfloat16 *b, long long n, cudaStream_t st);
cudaError_t fill_zero_bf16(__nv_bfloat16 *a, long long n, cudaStream_t st);

}  // namespace amk
