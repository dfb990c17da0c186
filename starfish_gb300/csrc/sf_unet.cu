// sf_unet.cu -- learned warm start for the Poisson solve: a 4-level U-Net in BF16 with
// FP32 accumulation, trained online on the GPU by this file's own forward and backward
// kernels.  (No reference counterpart: the Java reference solves every step from the
// previous potential.)
//
// The network maps the change of the solve's inputs since the last converged solve --
// charge density and electrode/boundary potentials -- to the change of the potential,
// on a grid coarsened by `down` (the change is smooth); the Poisson solve then starts
// from phi_prev + upsample(prediction) and still has to reach the same FP64 residual.
// Every converged solve yields one training pair, so the network learns from the
// simulation it accelerates.
//
// Convolutions are implicit GEMMs on the tensor cores with mma.sync m16n8k16 BF16
// (FP32 accumulate): forward (GEMM M = pixels, N = Cout, K = 9 Cin), backward data (the
// same kernel with flipped, transposed weights) and weight gradients (M = Cout, N = Cin,
// K = pixels, FP32 atomics across CTAs).  Activations are NHWC BF16.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>

#include "sf_internal.h"

using namespace sf;
typedef __nv_bfloat16 bf16;

namespace sf {
// the tensor-core (tcgen05) convolution, sf_conv_tc.cu
bool conv3x3_tc_supported(int H, int W, int Cin, int Cout, int out_C, int out_c0);
void conv3x3_tc(cudaStream_t s, const bf16* in, int H, int W, int Cin, const bf16* w, const float* bias, int Cout,
                bf16* out, int out_C, int out_c0, bool relu, int* err);
int conv3x3_tc_wait_test(cudaStream_t s);
}  // namespace sf

namespace {

constexpr int CONV_THREADS = 128;
constexpr int SEG = 64;  // pixels of one row segment per CTA tile

__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ unsigned ld_pair(const bf16* p) { return *reinterpret_cast<const unsigned*>(p); }

// 3x3 convolution, zero padding, stride 1.  in: H x W x Cin (NHWC), wt: Cout x 9 x Cin,
// out: H x W x out_C starting at channel out_c0.  NT = output channels per CTA.
// CTA tile: one row segment of SEG pixels x NT channels; warp w owns pixels [16w, 16w+16).
// Input channels are staged CI (16 or 32) at a time; the +8 padding of each shared row
// keeps the fragment loads free of bank conflicts (row strides of 12 or 20 words).
template <int NT, int CI>
__global__ void __launch_bounds__(CONV_THREADS) k_conv3x3(const bf16* __restrict__ in, int H, int W, int Cin,
                                                          const bf16* __restrict__ wt, const float* __restrict__ bias,
                                                          bf16* __restrict__ out, int out_C, int out_c0, int relu) {
  __shared__ __align__(16) bf16 s_in[SEG + 2][CI + 8];
  __shared__ __align__(16) bf16 s_w[NT][3][CI + 8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int x0 = blockIdx.x * SEG, y = blockIdx.y, co0 = blockIdx.z * NT;
  float acc[NT / 8][4];
#pragma unroll
  for (int n = 0; n < NT / 8; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
  for (int ky = 0; ky < 3; ky++) {
    const int yy = y + ky - 1;
    if (yy < 0 || yy >= H) continue;  // uniform over the CTA
    for (int ci0 = 0; ci0 < Cin; ci0 += CI) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < (SEG + 2) * (CI / 2); idx += CONV_THREADS) {
        const int pix = idx / (CI / 2), cp = idx % (CI / 2);
        const int xx = x0 - 1 + pix;
        unsigned v = 0u;
        if (xx >= 0 && xx < W) v = ld_pair(in + ((size_t)yy * W + xx) * Cin + ci0 + 2 * cp);
        *reinterpret_cast<unsigned*>(&s_in[pix][2 * cp]) = v;
      }
      for (int idx = threadIdx.x; idx < NT * 3 * (CI / 2); idx += CONV_THREADS) {
        const int co = idx / (3 * (CI / 2)), r = idx % (3 * (CI / 2));
        const int kx = r / (CI / 2), cp = r % (CI / 2);
        *reinterpret_cast<unsigned*>(&s_w[co][kx][2 * cp]) =
            ld_pair(wt + ((size_t)(co0 + co) * 9 + ky * 3 + kx) * Cin + ci0 + 2 * cp);
      }
      __syncthreads();
#pragma unroll
      for (int kx = 0; kx < 3; kx++) {
#pragma unroll
        for (int kk = 0; kk < CI; kk += 16) {
          unsigned a[4];
          const int p = 16 * w + g + kx;
          a[0] = *reinterpret_cast<const unsigned*>(&s_in[p][kk + 2 * t]);
          a[1] = *reinterpret_cast<const unsigned*>(&s_in[p + 8][kk + 2 * t]);
          a[2] = *reinterpret_cast<const unsigned*>(&s_in[p][kk + 2 * t + 8]);
          a[3] = *reinterpret_cast<const unsigned*>(&s_in[p + 8][kk + 2 * t + 8]);
#pragma unroll
          for (int n = 0; n < NT / 8; n++) {
            unsigned b[2];
            b[0] = *reinterpret_cast<const unsigned*>(&s_w[n * 8 + g][kx][kk + 2 * t]);
            b[1] = *reinterpret_cast<const unsigned*>(&s_w[n * 8 + g][kx][kk + 2 * t + 8]);
            mma_bf16(acc[n], a, b);
          }
        }
      }
    }
  }
  // epilogue: bias, ReLU, BF16 pairs
#pragma unroll
  for (int n = 0; n < NT / 8; n++) {
    const int co = co0 + n * 8 + 2 * t;
    const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int x = x0 + 16 * w + g + 8 * h;
      if (x >= W) continue;
      float v0 = acc[n][2 * h] + b0, v1 = acc[n][2 * h + 1] + b1;
      if (relu) {
        v0 = fmaxf(v0, 0.f);
        v1 = fmaxf(v1, 0.f);
      }
      *reinterpret_cast<__nv_bfloat162*>(out + ((size_t)y * W + x) * out_C + out_c0 + co) = __floats2bfloat162_rn(v0, v1);
    }
  }
}

// weight gradient of one tap (blockIdx.y = ky*3+kx) for a CO x CIT tile (blockIdx.z);
// row segments are distributed over blockIdx.x.  dW is FP32, accumulated atomically.
template <int CO, int CIT>
__global__ void __launch_bounds__(CONV_THREADS) k_conv3x3_wgrad(const bf16* __restrict__ gout, const bf16* __restrict__ in,
                                                                int H, int W, int Cin, int Cout, float* __restrict__ dW) {
  __shared__ __align__(16) bf16 s_g[CO][SEG + 8];    // [co][pixel]
  __shared__ __align__(16) bf16 s_x[CIT][SEG + 8];   // [ci][pixel]
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int tap = blockIdx.y, ky = tap / 3, kx = tap % 3;
  const int nci = Cin / CIT;
  const int co0 = (blockIdx.z / nci) * CO, ci0 = (blockIdx.z % nci) * CIT;
  const int segs_per_row = (W + SEG - 1) / SEG;
  const int nseg = H * segs_per_row;
  float acc[CIT / 8][4];
#pragma unroll
  for (int n = 0; n < CIT / 8; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
  const bool active = (w * 16) < CO;
  for (int s = blockIdx.x; s < nseg; s += gridDim.x) {
    const int y = s / segs_per_row, x0 = (s % segs_per_row) * SEG;
    const int yy = y + ky - 1;
    __syncthreads();
    for (int idx = threadIdx.x; idx < CO * SEG; idx += CONV_THREADS) {
      const int pix = idx / CO, co = idx % CO;
      const int x = x0 + pix;
      s_g[co][pix] = (x < W) ? gout[((size_t)y * W + x) * Cout + co0 + co] : __float2bfloat16(0.f);
    }
    for (int idx = threadIdx.x; idx < CIT * SEG; idx += CONV_THREADS) {
      const int pix = idx / CIT, ci = idx % CIT;
      const int xx = x0 + pix + kx - 1;
      const bool ok = (yy >= 0 && yy < H && xx >= 0 && xx < W && x0 + pix < W);
      s_x[ci][pix] = ok ? in[((size_t)yy * W + xx) * Cin + ci0 + ci] : __float2bfloat16(0.f);
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int kc = 0; kc < SEG / 16; kc++) {
        unsigned a[4];
        const int r = 16 * w + g;
        a[0] = *reinterpret_cast<const unsigned*>(&s_g[r][kc * 16 + 2 * t]);
        a[1] = *reinterpret_cast<const unsigned*>(&s_g[r + 8][kc * 16 + 2 * t]);
        a[2] = *reinterpret_cast<const unsigned*>(&s_g[r][kc * 16 + 2 * t + 8]);
        a[3] = *reinterpret_cast<const unsigned*>(&s_g[r + 8][kc * 16 + 2 * t + 8]);
#pragma unroll
        for (int n = 0; n < CIT / 8; n++) {
          unsigned b[2];
          b[0] = *reinterpret_cast<const unsigned*>(&s_x[n * 8 + g][kc * 16 + 2 * t]);
          b[1] = *reinterpret_cast<const unsigned*>(&s_x[n * 8 + g][kc * 16 + 2 * t + 8]);
          mma_bf16(acc[n], a, b);
        }
      }
    }
  }
  if (!active) return;
#pragma unroll
  for (int n = 0; n < CIT / 8; n++) {
    const int ci = ci0 + n * 8 + 2 * t;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int co = co0 + 16 * w + g + 8 * h;
      atomicAdd(&dW[((size_t)co * 9 + tap) * Cin + ci], acc[n][2 * h]);
      atomicAdd(&dW[((size_t)co * 9 + tap) * Cin + ci + 1], acc[n][2 * h + 1]);
    }
  }
}

// W'[ci][ky][kx][co] = W[co][2-ky][2-kx][ci]: weights of the backward-data convolution
__global__ void k_flip_weights(const bf16* __restrict__ w, int Cout, int Cin, bf16* __restrict__ wf) {
  const int n = Cout * 9 * Cin;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int ci = q % Cin, tap = (q / Cin) % 9, co = q / (9 * Cin);
    wf[((size_t)ci * 9 + (8 - tap)) * Cout + co] = w[q];
  }
}

// g *= (y > 0) for a ReLU output y; channel slice [c0, c0+C) of a C_total-wide tensor
__global__ void k_relu_grad(size_t npix, int C, const bf16* __restrict__ y, bf16* __restrict__ gr) {
  const size_t n = npix * C;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    if (!(__bfloat162float(y[q]) > 0.f)) gr[q] = __float2bfloat16(0.f);
}

__global__ void k_bias_grad(size_t npix, int C, const bf16* __restrict__ gr, float* __restrict__ db) {
  // one block per channel group of 32; threads stride over pixels
  const int c = blockIdx.y * 32 + (threadIdx.x & 31);
  if (c >= C) return;
  float s = 0.f;
  for (size_t p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); p < npix; p += (size_t)gridDim.x * (blockDim.x / 32))
    s += __bfloat162float(gr[p * C + c]);
  atomicAdd(&db[c], s);
}

// 2x2 average pooling and its adjoint
__global__ void k_pool(const bf16* __restrict__ in, int H, int W, int C, bf16* __restrict__ out) {
  const int Ho = H / 2, Wo = W / 2;
  const size_t n = (size_t)Ho * Wo * C;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int c = q % C;
    const size_t p = q / C;
    const int x = p % Wo, y = p / Wo;
    const size_t b = ((size_t)(2 * y) * W + 2 * x) * C + c;
    const float s = __bfloat162float(in[b]) + __bfloat162float(in[b + C]) + __bfloat162float(in[b + (size_t)W * C]) +
                    __bfloat162float(in[b + (size_t)W * C + C]);
    out[q] = __float2bfloat16(0.25f * s);
  }
}
__global__ void k_pool_grad(const bf16* __restrict__ gout, int H, int W, int C, bf16* __restrict__ gin, int accumulate) {
  const size_t n = (size_t)H * W * C;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int c = q % C;
    const size_t p = q / C;
    const int x = p % W, y = p / W;
    float v = 0.25f * __bfloat162float(gout[((size_t)(y / 2) * (W / 2) + x / 2) * C + c]);
    if (accumulate) v += __bfloat162float(gin[q]);
    gin[q] = __float2bfloat16(v);
  }
}

// nearest upsampling by 2 into channels [0, C) of a Ct-wide tensor, and its adjoint
__global__ void k_upsample(const bf16* __restrict__ in, int Hi, int Wi, int C, bf16* __restrict__ out, int Ct) {
  const int H = 2 * Hi, W = 2 * Wi;
  const size_t n = (size_t)H * W * C;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int c = q % C;
    const size_t p = q / C;
    const int x = p % W, y = p / W;
    out[p * Ct + c] = in[((size_t)(y / 2) * Wi + x / 2) * C + c];
  }
}
__global__ void k_upsample_grad(const bf16* __restrict__ gout, int Ct, int Hi, int Wi, int C, bf16* __restrict__ gin) {
  const size_t n = (size_t)Hi * Wi * C;
  const int W = 2 * Wi;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int c = q % C;
    const size_t p = q / C;
    const int x = p % Wi, y = p / Wi;
    const size_t b = ((size_t)(2 * y) * W + 2 * x) * Ct + c;
    const float s = __bfloat162float(gout[b]) + __bfloat162float(gout[b + Ct]) +
                    __bfloat162float(gout[b + (size_t)W * Ct]) + __bfloat162float(gout[b + (size_t)W * Ct + Ct]);
    gin[q] = __float2bfloat16(s);
  }
}

// copy channels: dst[p][c0 + c] = src[p][c], c < C (skip connection into a concat buffer),
// or the reverse with accumulate (its gradient back to the skip tensor)
__global__ void k_copy_channels(size_t npix, int C, const bf16* __restrict__ src, int Cs, int s0, bf16* __restrict__ dst,
                                int Cd, int d0, int accumulate) {
  const size_t n = npix * C;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int c = q % C;
    const size_t p = q / C;
    float v = __bfloat162float(src[p * Cs + s0 + c]);
    if (accumulate) v += __bfloat162float(dst[p * Cd + d0 + c]);
    dst[p * Cd + d0 + c] = __float2bfloat16(v);
  }
}

// 1x1 output head (C -> 1, FP32 out) and its gradients
__global__ void k_head(size_t npix, int C, const bf16* __restrict__ in, const float* __restrict__ w, const float* __restrict__ b,
                       float* __restrict__ out) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
    float s = b[0];
    for (int c = 0; c < C; c++) s += w[c] * __bfloat162float(in[p * C + c]);
    out[p] = s;
  }
}
__global__ void k_head_grad(size_t npix, int C, const bf16* __restrict__ in, const float* __restrict__ w,
                            const float* __restrict__ gout, bf16* __restrict__ gin, float* __restrict__ dw, float* __restrict__ db) {
  __shared__ float sw[64];
  __shared__ float sb;
  if (threadIdx.x < 64) sw[threadIdx.x] = 0.f;
  if (threadIdx.x == 0) sb = 0.f;
  __syncthreads();
  float lw[64];
  for (int c = 0; c < C; c++) lw[c] = 0.f;
  float lb = 0.f;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
    const float g = gout[p];
    lb += g;
    for (int c = 0; c < C; c++) {
      lw[c] += g * __bfloat162float(in[p * C + c]);
      gin[p * C + c] = __float2bfloat16(g * w[c]);
    }
  }
  for (int c = 0; c < C; c++) atomicAdd(&sw[c], lw[c]);
  atomicAdd(&sb, lb);
  __syncthreads();
  if (threadIdx.x < C) atomicAdd(&dw[threadIdx.x], sw[threadIdx.x]);
  if (threadIdx.x == 0) atomicAdd(db, sb);
}

// MSE loss over the network grid: gout = 2 (pred - target) / n, loss partial sums
__global__ void k_mse(size_t n, const float* __restrict__ pred, const float* __restrict__ target, float* __restrict__ gout,
                      float* __restrict__ loss) {
  float s = 0.f;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const float d = pred[p] - target[p];
    gout[p] = 2.f * d / (float)n;
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (float)n);
}

// Adam on FP32 master parameters, BF16 copies for the convolutions
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m, float* __restrict__ v,
                       float lr, float b1, float b2, float eps, float c1, float c2, bf16* __restrict__ p16) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const float g = gr[q];
    const float mm = b1 * m[q] + (1.f - b1) * g;
    const float vv = b2 * v[q] + (1.f - b2) * g * g;
    m[q] = mm;
    v[q] = vv;
    const float np = p[q] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
    p[q] = np;
    if (p16) p16[q] = __float2bfloat16(np);
  }
}

__global__ void k_f32_to_bf16(int n, const float* __restrict__ a, bf16* __restrict__ b) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) b[q] = __float2bfloat16(a[q]);
}

constexpr uint8_t NODE_FIXED = 1;  // node class of a Dirichlet node in the Poisson solve

// Per-sample normalisation.  The map (d rho, d bc) -> d phi is close to linear, so every
// pair is divided by its own scale
//   sigma = max |d bc| (fixed nodes) + k_rho * RMS(d rho),   k_rho = (L/4)^2 / eps
// (the potential a charge change of that RMS induces over a quarter of the domain), and
// the network predicts d phi / sigma; the warm start multiplies the prediction back.
// stats[0] = max |d bc| (float bits, non-negative so integer max orders them),
// stats[1] = sum d rho^2, stats[2] = max |bc|.
__global__ void k_unet_sigma_partial(size_t n, const double* __restrict__ rho, const double* __restrict__ rho_prev,
                                     const double* __restrict__ bc, const double* __restrict__ bc_prev,
                                     const uint8_t* __restrict__ type, unsigned* __restrict__ maxbits,
                                     double* __restrict__ sum2) {
  float mb = 0.f, ma = 0.f;
  double s2 = 0.0;
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < n; u += (size_t)gridDim.x * blockDim.x) {
    const double d = rho[u] - rho_prev[u];
    s2 += d * d;
    if (type[u] == NODE_FIXED) {
      mb = fmaxf(mb, (float)fabs(bc[u] - bc_prev[u]));
      ma = fmaxf(ma, (float)fabs(bc[u]));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mb = fmaxf(mb, __shfl_down_sync(0xffffffffu, mb, o));
    ma = fmaxf(ma, __shfl_down_sync(0xffffffffu, ma, o));
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&maxbits[0], __float_as_uint(mb));
    atomicMax(&maxbits[2], __float_as_uint(ma));
    atomicAdd(sum2, s2);
  }
}
__global__ void k_unet_sigma_final(size_t n, const unsigned* __restrict__ maxbits, const double* __restrict__ sum2,
                                   double k_rho, float* __restrict__ sigma) {
  const double s = (double)__uint_as_float(maxbits[0]) + k_rho * sqrt(*sum2 / (double)n);
  sigma[0] = (float)fmax(s, 1e-6);  // floor: 1 uV
}

// Network inputs from the solver state, per network pixel (X, Y) covering fine nodes
// [down X, down X + down) x [down Y, down Y + down):
//   0  k_rho * d rho / sigma, block mean (the particle noise of rho averages out)
//   1  d bc / sigma on fixed nodes, block mean
//   2  fraction of fixed nodes in the block
//   3  s_abs * phi_prev at node (down X, down Y) (the Boltzmann term makes d phi state dependent)
//   4..15 zero.
// target: d phi / sigma at node (down X, down Y).
struct InputArgs {
  int ni, nj, Hn, Wn, down;
  float k_rho, s_abs;
};
__global__ void k_unet_inputs(InputArgs a, const float* __restrict__ sigma, const double* __restrict__ rho,
                              const double* __restrict__ rho_prev, const double* __restrict__ bc,
                              const double* __restrict__ bc_prev, const uint8_t* __restrict__ type,
                              const double* __restrict__ phi, const double* __restrict__ phi_prev,
                              bf16* __restrict__ x, float* __restrict__ target) {
  const size_t n = (size_t)a.Hn * a.Wn;
  const double inv_sigma = 1.0 / (double)sigma[0];
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const int X = p % a.Wn, Y = p / a.Wn;
    double drho = 0, dbc = 0;
    int nfix = 0, cnt = 0;
    for (int dj = 0; dj < a.down; dj++) {
      const int j = a.down * Y + dj;
      if (j >= a.nj) break;
      for (int di = 0; di < a.down; di++) {
        const int i = a.down * X + di;
        if (i >= a.ni) break;
        const size_t u = (size_t)j * a.ni + i;
        drho += rho[u] - rho_prev[u];
        if (type[u] == NODE_FIXED) {
          dbc += bc[u] - bc_prev[u];
          nfix++;
        }
        cnt++;
      }
    }
    const size_t u0 = (size_t)(a.down * Y) * a.ni + a.down * X;
    bf16* xp = x + p * 16;
    xp[0] = __float2bfloat16((float)(a.k_rho * drho / cnt * inv_sigma));
    xp[1] = __float2bfloat16((float)(dbc / cnt * inv_sigma));
    xp[2] = __float2bfloat16((float)nfix / (float)cnt);
    xp[3] = __float2bfloat16((float)phi_prev[u0] * a.s_abs);
    for (int c = 4; c < 16; c++) xp[c] = __float2bfloat16(0.f);
    if (target) target[p] = (float)((phi[u0] - phi_prev[u0]) * inv_sigma);
  }
}

// phi = phi_prev + sigma * bilinear(prediction) on non-fixed nodes
__global__ void k_unet_apply(InputArgs a, const float* __restrict__ sigma, const float* __restrict__ pred,
                             const uint8_t* __restrict__ type, const double* __restrict__ phi_prev,
                             double* __restrict__ phi) {
  const size_t n = (size_t)a.ni * a.nj;
  const float sg = sigma[0];
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < n; u += (size_t)gridDim.x * blockDim.x) {
    if (type[u] == NODE_FIXED) continue;
    const int i = u % a.ni, j = u / a.ni;
    const float fx = (float)i / a.down, fy = (float)j / a.down;
    const int X = min((int)fx, a.Wn - 1), Y = min((int)fy, a.Hn - 1);
    const int X1 = min(X + 1, a.Wn - 1), Y1 = min(Y + 1, a.Hn - 1);
    const float wx = fminf(fx - X, 1.f), wy = fminf(fy - Y, 1.f);
    const float v = (1 - wx) * (1 - wy) * pred[(size_t)Y * a.Wn + X] + wx * (1 - wy) * pred[(size_t)Y * a.Wn + X1] +
                    wx * wy * pred[(size_t)Y1 * a.Wn + X1] + (1 - wx) * wy * pred[(size_t)Y1 * a.Wn + X];
    phi[u] = phi_prev[u] + (double)(sg * v);
  }
}

// ---- the network as a coarse correction inside the Poisson solve's PCG ------------
// Input of the correction for a linear residual r (FP32, the Newton system J e = r) and
// the Newton diagonal P, per network pixel covering down x down fine nodes:
//   0  r block mean / RMS(r)        1  fraction of fixed nodes        2  (L/4)^2 P block mean
// The network predicts e / s with s = (L/4)^2 RMS(r); the correction is s bilinear(pred)
// on the free nodes and zero on fixed ones.  RMS(r) comes from sum2 (sum of r^2 over the
// fine nodes).
struct PcArgs {
  int ni, nj, Hn, Wn, down;
  float L4sq;  // (L / 4)^2
};

__global__ void k_pc_sum2(size_t n, const float* __restrict__ r, double* __restrict__ sum2) {
  double s2 = 0.0;
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < n; u += (size_t)gridDim.x * blockDim.x) {
    const double v = r[u];
    s2 += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) s2 += __shfl_down_sync(0xffffffffu, s2, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(sum2, s2);
}

__global__ void k_pc_inputs(PcArgs a, const double* __restrict__ sum2, const float* __restrict__ r,
                            const float* __restrict__ P, const uint8_t* __restrict__ type, bf16* __restrict__ x) {
  const size_t n = (size_t)a.Hn * a.Wn;
  const float rms = (float)sqrt(*sum2 / ((double)a.ni * a.nj));
  const float inv = rms > 0.f ? 1.f / rms : 0.f;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const int X = p % a.Wn, Y = p / a.Wn;
    float rs = 0.f, ps = 0.f;
    int nfix = 0, cnt = 0;
    for (int dj = 0; dj < a.down; dj++) {
      const int j = a.down * Y + dj;
      if (j >= a.nj) break;
      for (int di = 0; di < a.down; di++) {
        const int i = a.down * X + di;
        if (i >= a.ni) break;
        const size_t u = (size_t)j * a.ni + i;
        rs += r[u];
        ps += P[u];
        nfix += type[u] == NODE_FIXED;
        cnt++;
      }
    }
    bf16* xp = x + p * 16;
    xp[0] = __float2bfloat16(rs / cnt * inv);
    xp[1] = __float2bfloat16((float)nfix / (float)cnt);
    xp[2] = __float2bfloat16(a.L4sq * ps / cnt);
    for (int c = 3; c < 16; c++) xp[c] = __float2bfloat16(0.f);
  }
}

// e = s bilinear(pred) on free nodes, 0 on fixed nodes
__global__ void k_pc_apply(PcArgs a, const double* __restrict__ sum2, const float* __restrict__ pred,
                           const uint8_t* __restrict__ type, float* __restrict__ e) {
  const size_t n = (size_t)a.ni * a.nj;
  const float s = a.L4sq * (float)sqrt(*sum2 / (double)n);
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < n; u += (size_t)gridDim.x * blockDim.x) {
    if (type[u] == NODE_FIXED) {
      e[u] = 0.f;
      continue;
    }
    const int i = u % a.ni, j = u / a.ni;
    const float fx = (float)i / a.down, fy = (float)j / a.down;
    const int X = min((int)fx, a.Wn - 1), Y = min((int)fy, a.Hn - 1);
    const int X1 = min(X + 1, a.Wn - 1), Y1 = min(Y + 1, a.Hn - 1);
    const float wx = fminf(fx - X, 1.f), wy = fminf(fy - Y, 1.f);
    const float v = (1 - wx) * (1 - wy) * pred[(size_t)Y * a.Wn + X] + wx * (1 - wy) * pred[(size_t)Y * a.Wn + X1] +
                    wx * wy * pred[(size_t)Y1 * a.Wn + X1] + (1 - wx) * wy * pred[(size_t)Y1 * a.Wn + X];
    e[u] = s * v;
  }
}

// training target of the correction: (phi_start - phi_end) / s at node (down X, down Y):
// the Newton correction the whole solve applied to its first residual
__global__ void k_pc_target(PcArgs a, const double* __restrict__ sum2, const double* __restrict__ phi_start,
                            const double* __restrict__ phi_end, float* __restrict__ target) {
  const size_t n = (size_t)a.Hn * a.Wn;
  const double s = (double)a.L4sq * sqrt(*sum2 / ((double)a.ni * a.nj));
  const double inv = s > 0 ? 1.0 / s : 0.0;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const int X = p % a.Wn, Y = p / a.Wn;
    const size_t u0 = (size_t)(a.down * Y) * a.ni + a.down * X;
    target[p] = (float)((phi_start[u0] - phi_end[u0]) * inv);
  }
}

}  // namespace

// ------------------------------------------------------------------------------------
// host: the network
// ------------------------------------------------------------------------------------
struct UConv {
  int cin, cout;
  size_t nw;
  bf16 *w16 = nullptr, *wflip = nullptr;
  float *w = nullptr, *b = nullptr, *gw = nullptr, *gb = nullptr, *mw = nullptr, *vw = nullptr, *mb = nullptr,
        *vb = nullptr;
};

struct UAct {
  bf16* p = nullptr;
  bf16* g = nullptr;  // gradient
  int H = 0, W = 0, C = 0;
  size_t npix() const { return (size_t)H * W; }
};

struct SfUnet {
  int levels = 4, base = 32, down = 1;
  int Hn = 0, Wn = 0;
  std::vector<UConv> convs;  // enc: 2 per level; dec: 2 per decoder level
  float *hw = nullptr, *hb = nullptr, *ghw = nullptr, *ghb = nullptr, *mhw = nullptr, *vhw = nullptr, *mhb = nullptr,
        *vhb = nullptr;
  UAct x;                       // input (16 ch)
  std::vector<UAct> enc;        // 2 per level
  std::vector<UAct> pool;       // levels-1
  std::vector<UAct> cat;        // levels-1 (decoder inputs)
  std::vector<UAct> dec;        // 2 per decoder level
  float *pred = nullptr, *target = nullptr, *gpred = nullptr, *loss = nullptr;
  std::vector<void*> allocs;
  cudaStream_t stream = nullptr;  // the context's stream (set-up copies and fills)
  int64_t samples = 0, steps = 0;
  int64_t pairs = 0;               // converged pairs seen while training
  int train_every = 1;             // one training step every train_every pairs
  int64_t used = 0, rejected = 0;  // predictions kept / rejected by the solve
  double last_loss = 0;
  float lr = 1e-3f;
  int iters_per_sample = 1;
  bool training = true;
  float s_abs = 0;  // scale of the phi_prev input: 1 / max |bc| at the first pair
  double k_rho = 0;  // (L/4)^2 / eps of the per-sample normalisation
  float* sigma = nullptr;      // per-sample scale (device)
  unsigned* maxbits = nullptr;  // reduction scratch: [0] max |d bc|, [2] max |bc| (float bits)
  double* sum2 = nullptr;       // reduction scratch: sum of d rho^2
  // solver state of the last converged solve
  double *phi_prev = nullptr, *rho_prev = nullptr, *bc_prev = nullptr;
  bool have_prev = false;
  int adam_t = 0;
  double train_ms = 0, infer_ms = 0;
  // coarse-correction mode: the first residual and Newton diagonal of the last solve and
  // its start potential (the training pair once it has converged), and the correction
  float *pc_r0 = nullptr, *pc_P0 = nullptr, *pc_e = nullptr;
  double* pc_phi0 = nullptr;
  double* pc_sum2 = nullptr;  // [0] sum r^2 of the current correction input, [1] of the saved r0
  bool pc_have = false;       // pc_r0 / pc_P0 / pc_phi0 hold the start of the last solve
  bool use_tc = true;         // tcgen05 convolutions where the shape allows
  int* tc_err = nullptr;      // device flag: a tensor-core convolution timed out
  int64_t tc_convs = 0;       // convolutions run on the tcgen05 path
};

static void* ualloc(SfUnet* u, size_t bytes) {
  void* p = nullptr;
  SF_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
  zero_wait(p, std::max<size_t>(bytes, 16), u->stream);
  u->allocs.push_back(p);
  return p;
}

static UAct make_act(SfUnet* u, int H, int W, int C) {
  UAct a;
  a.H = H;
  a.W = W;
  a.C = C;
  a.p = (bf16*)ualloc(u, sizeof(bf16) * (size_t)H * W * C);
  a.g = (bf16*)ualloc(u, sizeof(bf16) * (size_t)H * W * C);
  return a;
}

static UConv make_conv(SfUnet* u, int cin, int cout, std::mt19937& rng) {
  UConv c;
  c.cin = cin;
  c.cout = cout;
  c.nw = (size_t)cout * 9 * cin;
  std::vector<float> h(c.nw);
  // He initialisation over the 9 * fan-in inputs
  std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (9.f * cin)));
  for (auto& v : h) v = nd(rng);
  c.w = (float*)ualloc(u, 4 * c.nw);
  c.gw = (float*)ualloc(u, 4 * c.nw);
  c.mw = (float*)ualloc(u, 4 * c.nw);
  c.vw = (float*)ualloc(u, 4 * c.nw);
  c.b = (float*)ualloc(u, 4 * cout);
  c.gb = (float*)ualloc(u, 4 * cout);
  c.mb = (float*)ualloc(u, 4 * cout);
  c.vb = (float*)ualloc(u, 4 * cout);
  c.w16 = (bf16*)ualloc(u, 2 * c.nw);
  c.wflip = (bf16*)ualloc(u, 2 * c.nw);
  copy_wait(c.w, h.data(), 4 * c.nw, cudaMemcpyHostToDevice, u->stream);
  return c;
}

static int ew_grid(sf_ctx* ctx, size_t n) { return grid_for((int64_t)std::min<size_t>(n, 1u << 30), 256, ctx->num_sms * 8); }

// Forward (and backward-data) 3x3 convolution: on the tcgen05 tensor cores for the
// shapes sf_conv_tc.cu takes (grid rows of 16, 32, 64 or a multiple of 128 nodes), else on
// mma.sync.
static void conv_fwd(sf_ctx* ctx, const bf16* in, int H, int W, int Cin, const bf16* w16, const float* bias, int Cout,
                     bf16* out, int out_C, int out_c0, bool relu) {
  SF_REQUIRE(Cin % 16 == 0 && Cout % 16 == 0, SF_ERR_ARG, "U-Net channels must be multiples of 16");
  SfUnet* u = ctx->unet;
  if (u && u->use_tc && conv3x3_tc_supported(H, W, Cin, Cout, out_C, out_c0)) {
    conv3x3_tc(ctx->stream, in, H, W, Cin, w16, bias, Cout, out, out_C, out_c0, relu, u->tc_err);
    ctx->launches++;
    u->tc_convs++;
    return;
  }
  const int NT = Cout % 64 == 0 ? 64 : (Cout % 32 == 0 ? 32 : 16);  // must divide Cout
  const bool ci32 = Cin % 32 == 0;
  dim3 grid((W + SEG - 1) / SEG, H, Cout / NT);
  cudaStream_t s = ctx->stream;
  const int r = relu ? 1 : 0;
#define CONV(nt, ci) k_conv3x3<nt, ci><<<grid, CONV_THREADS, 0, s>>>(in, H, W, Cin, w16, bias, out, out_C, out_c0, r)
  if (NT == 64) {
    if (ci32) CONV(64, 32); else CONV(64, 16);
  } else if (NT == 32) {
    if (ci32) CONV(32, 32); else CONV(32, 16);
  } else {
    if (ci32) CONV(16, 32); else CONV(16, 16);
  }
#undef CONV
  ctx->launches++;
}

// After a stream synchronisation: a tensor-core convolution whose pipeline wait ran out
// left its output incomplete; report it (and clear the flag for the next call).
static void check_tc(sf_ctx* ctx, SfUnet* u) {
  int e = 0;
  copy_wait(&e, u->tc_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e) {
    zero_wait(u->tc_err, sizeof(int), ctx->stream);
    SF_REQUIRE(false, SF_ERR_TIMEOUT, "a tensor-core convolution of the U-Net timed out");
  }
}

static void conv_wgrad(sf_ctx* ctx, const bf16* gout, const bf16* in, int H, int W, int Cin, int Cout, float* dW) {
  // tile widths must divide the channel counts (concatenations give 96, 192, 384)
  const int CO = Cout % 64 == 0 ? 64 : (Cout % 32 == 0 ? 32 : 16);
  const int CIT = Cin % 64 == 0 ? 64 : (Cin % 32 == 0 ? 32 : 16);
  const int tiles = (Cout / CO) * (Cin / CIT);
  const int segs = H * ((W + SEG - 1) / SEG);
  const int gx = std::max(1, std::min(segs, (ctx->num_sms * 4) / std::max(1, 9 * tiles / 8 + 1)));
  dim3 grid(gx, 9, tiles);
  cudaStream_t s = ctx->stream;
#define WG(a, b)                                                                                                  \
  if (CO == a && CIT == b) {                                                                                      \
    k_conv3x3_wgrad<a, b><<<grid, CONV_THREADS, 0, s>>>(gout, in, H, W, Cin, Cout, dW);                           \
    ctx->launches++;                                                                                              \
    return;                                                                                                       \
  }
  WG(64, 64) WG(64, 32) WG(64, 16) WG(32, 64) WG(32, 32) WG(32, 16) WG(16, 64) WG(16, 32) WG(16, 16)
#undef WG
  SF_REQUIRE(false, SF_ERR_ARG, "unsupported U-Net channel count");
}

static void unet_build(sf_ctx* ctx, SfUnet* u, uint64_t seed) {
  std::mt19937 rng((uint32_t)seed);
  const int L = u->levels;
  std::vector<int> C(L);
  for (int l = 0; l < L; l++) C[l] = u->base << l;
  int cin = 16;
  for (int l = 0; l < L; l++) {
    u->convs.push_back(make_conv(u, cin, C[l], rng));
    u->convs.push_back(make_conv(u, C[l], C[l], rng));
    cin = C[l];
  }
  for (int l = L - 2; l >= 0; l--) {
    u->convs.push_back(make_conv(u, C[l + 1] + C[l], C[l], rng));
    u->convs.push_back(make_conv(u, C[l], C[l], rng));
  }
  // output head (C[0] -> 1), small initial weights
  std::vector<float> hw(C[0]);
  std::normal_distribution<float> nd(0.f, 0.01f);
  for (auto& v : hw) v = nd(rng);
  u->hw = (float*)ualloc(u, 4 * C[0]);
  u->hb = (float*)ualloc(u, 4);
  u->ghw = (float*)ualloc(u, 4 * C[0]);
  u->ghb = (float*)ualloc(u, 4);
  u->mhw = (float*)ualloc(u, 4 * C[0]);
  u->vhw = (float*)ualloc(u, 4 * C[0]);
  u->mhb = (float*)ualloc(u, 4);
  u->vhb = (float*)ualloc(u, 4);
  copy_wait(u->hw, hw.data(), 4 * C[0], cudaMemcpyHostToDevice, u->stream);
  // activations
  u->x = make_act(u, u->Hn, u->Wn, 16);
  int H = u->Hn, W = u->Wn;
  for (int l = 0; l < L; l++) {
    u->enc.push_back(make_act(u, H, W, C[l]));
    u->enc.push_back(make_act(u, H, W, C[l]));
    if (l < L - 1) u->pool.push_back(make_act(u, H / 2, W / 2, C[l]));
    H /= 2;
    W /= 2;
  }
  for (int l = L - 2; l >= 0; l--) {
    const int Hl = u->Hn >> l, Wl = u->Wn >> l;
    u->cat.push_back(make_act(u, Hl, Wl, C[l + 1] + C[l]));
    u->dec.push_back(make_act(u, Hl, Wl, C[l]));
    u->dec.push_back(make_act(u, Hl, Wl, C[l]));
  }
  const size_t np = (size_t)u->Hn * u->Wn;
  u->pred = (float*)ualloc(u, 4 * np);
  u->target = (float*)ualloc(u, 4 * np);
  u->gpred = (float*)ualloc(u, 4 * np);
  u->loss = (float*)ualloc(u, 4);
  for (auto& c : u->convs) {
    k_f32_to_bf16<<<ew_grid(ctx, c.nw), 256, 0, ctx->stream>>>((int)c.nw, c.w, c.w16);
    ctx->launches++;
  }
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
}

// forward pass from u->x to u->pred
static void unet_forward(sf_ctx* ctx, SfUnet* u) {
  cudaStream_t s = ctx->stream;
  const int L = u->levels;
  const bf16* in = u->x.p;
  int cin = 16;
  for (int l = 0; l < L; l++) {
    UConv& c0 = u->convs[2 * l];
    UConv& c1 = u->convs[2 * l + 1];
    UAct& a0 = u->enc[2 * l];
    UAct& a1 = u->enc[2 * l + 1];
    conv_fwd(ctx, in, a0.H, a0.W, cin, c0.w16, c0.b, c0.cout, a0.p, a0.C, 0, true);
    conv_fwd(ctx, a0.p, a1.H, a1.W, a0.C, c1.w16, c1.b, c1.cout, a1.p, a1.C, 0, true);
    if (l < L - 1) {
      UAct& pl = u->pool[l];
      k_pool<<<ew_grid(ctx, pl.npix() * pl.C), 256, 0, s>>>(a1.p, a1.H, a1.W, a1.C, pl.p);
      ctx->launches++;
      in = pl.p;
      cin = pl.C;
    }
  }
  const bf16* below = u->enc[2 * (L - 1) + 1].p;
  int cb = u->enc[2 * (L - 1) + 1].C;
  for (int k = 0; k < L - 1; k++) {
    const int l = L - 2 - k;
    UAct& ct = u->cat[k];
    UAct& skip = u->enc[2 * l + 1];
    k_upsample<<<ew_grid(ctx, ct.npix() * cb), 256, 0, s>>>(below, ct.H / 2, ct.W / 2, cb, ct.p, ct.C);
    k_copy_channels<<<ew_grid(ctx, ct.npix() * skip.C), 256, 0, s>>>(ct.npix(), skip.C, skip.p, skip.C, 0, ct.p, ct.C, cb, 0);
    ctx->launches += 2;
    UConv& c0 = u->convs[2 * L + 2 * k];
    UConv& c1 = u->convs[2 * L + 2 * k + 1];
    UAct& d0 = u->dec[2 * k];
    UAct& d1 = u->dec[2 * k + 1];
    conv_fwd(ctx, ct.p, ct.H, ct.W, ct.C, c0.w16, c0.b, c0.cout, d0.p, d0.C, 0, true);
    conv_fwd(ctx, d0.p, d1.H, d1.W, d0.C, c1.w16, c1.b, c1.cout, d1.p, d1.C, 0, true);
    below = d1.p;
    cb = d1.C;
  }
  UAct& last = u->dec[2 * (L - 2) + 1];
  k_head<<<ew_grid(ctx, last.npix()), 256, 0, s>>>(last.npix(), last.C, last.p, u->hw, u->hb, u->pred);
  ctx->launches++;
}

// backward pass from u->gpred; parameter gradients into gw/gb (zeroed here)
static void unet_backward(sf_ctx* ctx, SfUnet* u) {
  cudaStream_t s = ctx->stream;
  const int L = u->levels;
  for (auto& c : u->convs) {
    SF_CUDA(cudaMemsetAsync(c.gw, 0, 4 * c.nw, s));
    SF_CUDA(cudaMemsetAsync(c.gb, 0, 4 * c.cout, s));
    k_flip_weights<<<ew_grid(ctx, c.nw), 256, 0, s>>>(c.w16, c.cout, c.cin, c.wflip);
    ctx->launches++;
  }
  SF_CUDA(cudaMemsetAsync(u->ghw, 0, 4 * u->base, s));
  SF_CUDA(cudaMemsetAsync(u->ghb, 0, 4, s));
  UAct& last = u->dec[2 * (L - 2) + 1];
  k_head_grad<<<ctx->num_sms * 2, 256, 0, s>>>(last.npix(), last.C, last.p, u->hw, u->gpred, last.g, u->ghw, u->ghb);
  ctx->launches++;
  // conv backward helper: g of output (already ReLU-masked) -> weight grads and g of input
  auto conv_bwd = [&](UConv& c, UAct& out, const bf16* in_p, int in_C, bf16* in_g, int H, int W) {
    k_relu_grad<<<ew_grid(ctx, out.npix() * out.C), 256, 0, s>>>(out.npix(), out.C, out.p, out.g);
    k_bias_grad<<<dim3(ctx->num_sms, (out.C + 31) / 32), 256, 0, s>>>(out.npix(), out.C, out.g, c.gb);
    ctx->launches += 2;
    conv_wgrad(ctx, out.g, in_p, H, W, in_C, c.cout, c.gw);
    if (in_g) conv_fwd(ctx, out.g, H, W, c.cout, c.wflip, nullptr, in_C, in_g, in_C, 0, false);
  };
  // decoder
  for (int k = L - 2; k >= 0; k--) {
    const int l = L - 2 - k;
    UAct& ct = u->cat[k];
    UAct& d0 = u->dec[2 * k];
    UAct& d1 = u->dec[2 * k + 1];
    UConv& c0 = u->convs[2 * L + 2 * k];
    UConv& c1 = u->convs[2 * L + 2 * k + 1];
    conv_bwd(c1, d1, d0.p, d0.C, d0.g, d1.H, d1.W);
    conv_bwd(c0, d0, ct.p, ct.C, ct.g, d0.H, d0.W);
    // split the concat gradient: upsampled part -> below, skip part -> encoder output
    UAct& skip = u->enc[2 * l + 1];
    UAct& below = (k == 0) ? u->enc[2 * (L - 1) + 1] : u->dec[2 * (k - 1) + 1];
    const int cb = ct.C - skip.C;
    k_upsample_grad<<<ew_grid(ctx, below.npix() * cb), 256, 0, s>>>(ct.g, ct.C, below.H, below.W, cb, below.g);
    k_copy_channels<<<ew_grid(ctx, skip.npix() * skip.C), 256, 0, s>>>(skip.npix(), skip.C, ct.g, ct.C, cb, skip.g, skip.C,
                                                                       0, 0);
    ctx->launches += 2;
  }
  // encoder (the skip gradients were written first, the pooled path adds to them)
  for (int l = L - 1; l >= 0; l--) {
    UAct& a0 = u->enc[2 * l];
    UAct& a1 = u->enc[2 * l + 1];
    UConv& c0 = u->convs[2 * l];
    UConv& c1 = u->convs[2 * l + 1];
    conv_bwd(c1, a1, a0.p, a0.C, a0.g, a1.H, a1.W);
    const bf16* in_p = (l == 0) ? u->x.p : u->pool[l - 1].p;
    const int in_C = (l == 0) ? 16 : u->pool[l - 1].C;
    bf16* in_g = (l == 0) ? nullptr : u->pool[l - 1].g;
    conv_bwd(c0, a0, in_p, in_C, in_g, a0.H, a0.W);
    if (l > 0) {
      UAct& pl = u->pool[l - 1];
      UAct& prev = u->enc[2 * (l - 1) + 1];
      k_pool_grad<<<ew_grid(ctx, prev.npix() * prev.C), 256, 0, s>>>(pl.g, prev.H, prev.W, prev.C, prev.g, 1);
      ctx->launches++;
    }
  }
}

static void unet_adam(sf_ctx* ctx, SfUnet* u) {
  cudaStream_t s = ctx->stream;
  u->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)u->adam_t)), c2 = 1.f / (1.f - std::pow(b2, (float)u->adam_t));
  for (auto& c : u->convs) {
    k_adam<<<ew_grid(ctx, c.nw), 256, 0, s>>>((int)c.nw, c.w, c.gw, c.mw, c.vw, u->lr, b1, b2, eps, c1, c2, c.w16);
    k_adam<<<1, 256, 0, s>>>(c.cout, c.b, c.gb, c.mb, c.vb, u->lr, b1, b2, eps, c1, c2, nullptr);
    ctx->launches += 2;
  }
  k_adam<<<1, 256, 0, s>>>(u->base, u->hw, u->ghw, u->mhw, u->vhw, u->lr, b1, b2, eps, c1, c2, nullptr);
  k_adam<<<1, 32, 0, s>>>(1, u->hb, u->ghb, u->mhb, u->vhb, u->lr, b1, b2, eps, c1, c2, nullptr);
  ctx->launches += 2;
}

// one training step on the current (x, target); returns the loss before the update
static double unet_train_step(sf_ctx* ctx, SfUnet* u) {
  cudaStream_t s = ctx->stream;
  unet_forward(ctx, u);
  const size_t np = (size_t)u->Hn * u->Wn;
  SF_CUDA(cudaMemsetAsync(u->loss, 0, 4, s));
  k_mse<<<ew_grid(ctx, np), 256, 0, s>>>(np, u->pred, u->target, u->gpred, u->loss);
  ctx->launches++;
  unet_backward(ctx, u);
  unet_adam(ctx, u);
  float l = 0;
  SF_CUDA(cudaMemcpyAsync(&l, u->loss, 4, cudaMemcpyDeviceToHost, s));
  SF_CUDA(cudaStreamSynchronize(s));
  u->steps++;
  return l;
}

// ------------------------------------------------------------------------------------
// hooks used by the Poisson solve (sf_poisson.cu) and the C ABI
// ------------------------------------------------------------------------------------
void sf_unet_destroy_internal(sf_ctx* ctx) {
  SfUnet* u = ctx->unet;
  if (!u) return;
  for (void* p : u->allocs) cudaFree(p);
  delete u;
  ctx->unet = nullptr;
}

static InputArgs input_args(sf_ctx* ctx, SfUnet* u) {
  InputArgs a;
  a.ni = ctx->ni;
  a.nj = ctx->nj;
  a.Hn = u->Hn;
  a.Wn = u->Wn;
  a.down = u->down;
  a.k_rho = (float)u->k_rho;
  a.s_abs = u->s_abs;
  return a;
}

// sigma of the pair (rho, bc) against the remembered state, on the stream
static void unet_sigma(sf_ctx* ctx, SfUnet* u, const double* rho, const double* bc, const uint8_t* type) {
  cudaStream_t s = ctx->stream;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  SF_CUDA(cudaMemsetAsync(u->maxbits, 0, 4 * sizeof(unsigned), s));
  SF_CUDA(cudaMemsetAsync(u->sum2, 0, sizeof(double), s));
  k_unet_sigma_partial<<<ew_grid(ctx, nn), 256, 0, s>>>(nn, rho, u->rho_prev, bc, u->bc_prev, type, u->maxbits,
                                                       u->sum2);
  k_unet_sigma_final<<<1, 1, 0, s>>>(nn, u->maxbits, u->sum2, u->k_rho, u->sigma);
  ctx->launches += 2;
}

void sf_unet_after_solve(sf_ctx* ctx, const double* phi, const double* rho, const double* bc, const uint8_t* type,
                         double eps) {
  SfUnet* u = ctx->unet;
  if (!u) return;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  cudaStream_t s = ctx->stream;
  const double L = std::min((ctx->ni - 1) * ctx->dh[0], (ctx->nj - 1) * ctx->dh[1]) / 4;
  u->k_rho = L * L / eps;
  if (u->have_prev && u->training && (u->pairs++ % u->train_every) == 0) {
    cudaEvent_t e0, e1;
    SF_CUDA(cudaEventCreate(&e0));
    SF_CUDA(cudaEventCreate(&e1));
    SF_CUDA(cudaEventRecord(e0, s));
    unet_sigma(ctx, u, rho, bc, type);
    if (u->s_abs == 0.f) {
      // scale of the phi_prev input, fixed at the first pair
      unsigned mb[4];
      SF_CUDA(cudaMemcpyAsync(mb, u->maxbits, sizeof(mb), cudaMemcpyDeviceToHost, s));
      SF_CUDA(cudaStreamSynchronize(s));
      float ma;
      std::memcpy(&ma, &mb[2], 4);
      u->s_abs = 1.f / std::max(ma, 1.f);
    }
    const InputArgs a = input_args(ctx, u);
    k_unet_inputs<<<ew_grid(ctx, (size_t)u->Hn * u->Wn), 256, 0, s>>>(a, u->sigma, rho, u->rho_prev, bc, u->bc_prev,
                                                                       type, phi, u->phi_prev, u->x.p, u->target);
    ctx->launches++;
    double l = 0;
    for (int k = 0; k < u->iters_per_sample; k++) l = unet_train_step(ctx, u);
    SF_CUDA(cudaEventRecord(e1, s));
    SF_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    u->train_ms += ms;
    u->last_loss = l;
    u->samples++;
    check_tc(ctx, u);
  }
  SF_CUDA(cudaMemcpyAsync(u->phi_prev, phi, 8 * nn, cudaMemcpyDeviceToDevice, s));
  SF_CUDA(cudaMemcpyAsync(u->rho_prev, rho, 8 * nn, cudaMemcpyDeviceToDevice, s));
  SF_CUDA(cudaMemcpyAsync(u->bc_prev, bc, 8 * nn, cudaMemcpyDeviceToDevice, s));
  u->have_prev = true;
}

bool sf_unet_warm_start(sf_ctx* ctx, double* phi, const double* rho, const double* bc, const uint8_t* type) {
  SfUnet* u = ctx->unet;
  if (!u || !u->have_prev || u->samples == 0) return false;
  cudaStream_t s = ctx->stream;
  unet_sigma(ctx, u, rho, bc, type);
  const InputArgs a = input_args(ctx, u);
  k_unet_inputs<<<ew_grid(ctx, (size_t)u->Hn * u->Wn), 256, 0, s>>>(a, u->sigma, rho, u->rho_prev, bc, u->bc_prev,
                                                                     type, nullptr, u->phi_prev, u->x.p, nullptr);
  ctx->launches++;
  unet_forward(ctx, u);
  k_unet_apply<<<ew_grid(ctx, (size_t)ctx->ni * ctx->nj), 256, 0, s>>>(a, u->sigma, u->pred, type, u->phi_prev, phi);
  ctx->launches++;
  u->used++;
  return true;
}

static PcArgs pc_args(sf_ctx* ctx, SfUnet* u) {
  PcArgs a;
  a.ni = ctx->ni;
  a.nj = ctx->nj;
  a.Hn = u->Hn;
  a.Wn = u->Wn;
  a.down = u->down;
  const double L = std::min((ctx->ni - 1) * ctx->dh[0], (ctx->nj - 1) * ctx->dh[1]) / 4;
  a.L4sq = (float)(L * L);
  return a;
}

static void pc_buffers(sf_ctx* ctx, SfUnet* u) {
  if (u->pc_e) return;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  u->pc_r0 = (float*)ualloc(u, 4 * nn);
  u->pc_P0 = (float*)ualloc(u, 4 * nn);
  u->pc_e = (float*)ualloc(u, 4 * nn);
  u->pc_phi0 = (double*)ualloc(u, 8 * nn);
  u->pc_sum2 = (double*)ualloc(u, 2 * sizeof(double));
}

// Launches the network's correction e for the residual r (only launches: the Newton step
// that calls it is captured as a CUDA graph).  e lives in the network's buffer, which the
// first use allocates: that first use happens at the start of a solve in this mode
// (sf_unet_coarse_start), before any capture.
float* sf_unet_coarse_correction(sf_ctx* ctx, const float* r, const float* P, const uint8_t* type) {
  SfUnet* u = ctx->unet;
  pc_buffers(ctx, u);
  cudaStream_t s = ctx->stream;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  const PcArgs a = pc_args(ctx, u);
  SF_CUDA(cudaMemsetAsync(u->pc_sum2, 0, sizeof(double), s));
  k_pc_sum2<<<ew_grid(ctx, nn), 256, 0, s>>>(nn, r, u->pc_sum2);
  k_pc_inputs<<<ew_grid(ctx, (size_t)u->Hn * u->Wn), 256, 0, s>>>(a, u->pc_sum2, r, P, type, u->x.p);
  unet_forward(ctx, u);
  k_pc_apply<<<ew_grid(ctx, nn), 256, 0, s>>>(a, u->pc_sum2, u->pred, type, u->pc_e);
  ctx->launches += 3;
  return u->pc_e;
}

// The start of a solve in coarse-correction mode: its first residual, Newton diagonal and
// potential, kept for the training pair the converged solve makes.
void sf_unet_coarse_start(sf_ctx* ctx, const float* r0, const float* P0, const double* phi0) {
  SfUnet* u = ctx->unet;
  pc_buffers(ctx, u);
  cudaStream_t s = ctx->stream;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  SF_CUDA(cudaMemcpyAsync(u->pc_r0, r0, 4 * nn, cudaMemcpyDeviceToDevice, s));
  SF_CUDA(cudaMemcpyAsync(u->pc_P0, P0, 4 * nn, cudaMemcpyDeviceToDevice, s));
  SF_CUDA(cudaMemcpyAsync(u->pc_phi0, phi0, 8 * nn, cudaMemcpyDeviceToDevice, s));
  u->pc_have = true;
}

// After a converged solve in coarse-correction mode (outside the solve's timing): one
// training step on (first residual, first Newton diagonal) -> the whole correction the
// solve applied, phi_start - phi_end.
void sf_unet_coarse_train(sf_ctx* ctx, const double* phi_end, const uint8_t* type) {
  SfUnet* u = ctx->unet;
  if (!u || !u->pc_have || !u->training) return;
  u->pc_have = false;
  cudaStream_t s = ctx->stream;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  const PcArgs a = pc_args(ctx, u);
  cudaEvent_t e0, e1;
  SF_CUDA(cudaEventCreate(&e0));
  SF_CUDA(cudaEventCreate(&e1));
  SF_CUDA(cudaEventRecord(e0, s));
  SF_CUDA(cudaMemsetAsync(u->pc_sum2 + 1, 0, sizeof(double), s));
  k_pc_sum2<<<ew_grid(ctx, nn), 256, 0, s>>>(nn, u->pc_r0, u->pc_sum2 + 1);
  k_pc_inputs<<<ew_grid(ctx, (size_t)u->Hn * u->Wn), 256, 0, s>>>(a, u->pc_sum2 + 1, u->pc_r0, u->pc_P0, type, u->x.p);
  k_pc_target<<<ew_grid(ctx, (size_t)u->Hn * u->Wn), 256, 0, s>>>(a, u->pc_sum2 + 1, u->pc_phi0, phi_end, u->target);
  ctx->launches += 3;
  double l = 0;
  for (int k = 0; k < u->iters_per_sample; k++) l = unet_train_step(ctx, u);
  SF_CUDA(cudaEventRecord(e1, s));
  SF_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  u->train_ms += ms;
  u->last_loss = l;
  u->samples++;
  check_tc(ctx, u);
}

bool sf_unet_coarse_ready(const sf_ctx* ctx) { return ctx->unet && ctx->unet->samples > 0; }

void sf_unet_reject(sf_ctx* ctx, double* phi) {
  SfUnet* u = ctx->unet;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  SF_CUDA(cudaMemcpyAsync(phi, u->phi_prev, 8 * nn, cudaMemcpyDeviceToDevice, ctx->stream));
  u->used--;
  u->rejected++;
}

extern "C" {

int sf_unet_init(sf_ctx* ctx, int32_t base_channels, int32_t down, uint64_t seed) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null context");
  SF_REQUIRE(base_channels == 16 || base_channels == 32, SF_ERR_ARG, "base channels must be 16 or 32");
  SF_REQUIRE(down >= 1 && down <= 8, SF_ERR_ARG, "down must be in 1..8");
  SF_CUDA(cudaSetDevice(ctx->device));
  sf_unet_destroy_internal(ctx);
  SfUnet* u = new SfUnet();
  ctx->unet = u;
  u->stream = ctx->stream;
  u->base = base_channels;
  u->down = down;
  u->Wn = (ctx->ni - 1) / down;
  u->Hn = (ctx->nj - 1) / down;
  SF_REQUIRE(u->Wn % 8 == 0 && u->Hn % 8 == 0 && u->Wn >= 16 && u->Hn >= 16, SF_ERR_ARG,
             "network grid (n-1)/down must be a multiple of 8 and >= 16 in both directions");
  unet_build(ctx, u, seed);
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  u->phi_prev = (double*)ualloc(u, 8 * nn);
  u->sigma = (float*)ualloc(u, sizeof(float));
  u->maxbits = (unsigned*)ualloc(u, 4 * sizeof(unsigned));
  u->sum2 = (double*)ualloc(u, sizeof(double));
  u->rho_prev = (double*)ualloc(u, 8 * nn);
  u->bc_prev = (double*)ualloc(u, 8 * nn);
  u->tc_err = (int*)ualloc(u, sizeof(int));
  SF_API_END(ctx)
}

int sf_unet_set_training(sf_ctx* ctx, int32_t on, double lr, int32_t iters_per_sample, int32_t every) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && ctx->unet, SF_ERR_STATE, "no U-Net (sf_unet_init)");
  SF_REQUIRE(lr > 0 && iters_per_sample >= 1 && every >= 1, SF_ERR_ARG, "bad training parameters");
  ctx->unet->training = on != 0;
  ctx->unet->lr = (float)lr;
  ctx->unet->iters_per_sample = iters_per_sample;
  ctx->unet->train_every = every;
  SF_API_END(ctx)
}

int sf_unet_stats(sf_ctx* ctx, double* last_loss, int64_t* samples, double* train_ms, int64_t* used,
                  int64_t* rejected) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && ctx->unet, SF_ERR_STATE, "no U-Net (sf_unet_init)");
  if (last_loss) *last_loss = ctx->unet->last_loss;
  if (samples) *samples = ctx->unet->samples;
  if (train_ms) *train_ms = ctx->unet->train_ms;
  if (used) *used = ctx->unet->used;
  if (rejected) *rejected = ctx->unet->rejected;
  SF_API_END(ctx)
}

// Gradient checking entry points: run the network on a given input (Hn*Wn*16 floats,
// NHWC) and return the prediction; with dpred given, also backpropagate and return the
// parameter gradients flattened in layer order (conv w, conv b, ..., head w, head b).
int sf_unet_debug(sf_ctx* ctx, const float* x, const float* dpred, float* pred, float* grads, int64_t* nparams) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && ctx->unet, SF_ERR_STATE, "no U-Net (sf_unet_init)");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfUnet* u = ctx->unet;
  cudaStream_t s = ctx->stream;
  const size_t np = (size_t)u->Hn * u->Wn;
  int64_t total = 0;
  for (auto& c : u->convs) total += (int64_t)c.nw + c.cout;
  total += u->base + 1;
  if (nparams) *nparams = total;
  if (!x) return SF_OK;
  std::vector<bf16> hx(np * 16);
  for (size_t q = 0; q < np * 16; q++) hx[q] = __float2bfloat16(x[q]);
  SF_CUDA(cudaMemcpyAsync(u->x.p, hx.data(), 2 * np * 16, cudaMemcpyHostToDevice, s));
  unet_forward(ctx, u);
  if (pred) SF_CUDA(cudaMemcpyAsync(pred, u->pred, 4 * np, cudaMemcpyDeviceToHost, s));
  if (dpred && grads) {
    SF_CUDA(cudaMemcpyAsync(u->gpred, dpred, 4 * np, cudaMemcpyHostToDevice, s));
    unet_backward(ctx, u);
    int64_t off = 0;
    for (auto& c : u->convs) {
      SF_CUDA(cudaMemcpyAsync(grads + off, c.gw, 4 * c.nw, cudaMemcpyDeviceToHost, s));
      off += (int64_t)c.nw;
      SF_CUDA(cudaMemcpyAsync(grads + off, c.gb, 4 * c.cout, cudaMemcpyDeviceToHost, s));
      off += c.cout;
    }
    SF_CUDA(cudaMemcpyAsync(grads + off, u->ghw, 4 * u->base, cudaMemcpyDeviceToHost, s));
    off += u->base;
    SF_CUDA(cudaMemcpyAsync(grads + off, u->ghb, 4, cudaMemcpyDeviceToHost, s));
  }
  SF_CUDA(cudaGetLastError());
  SF_CUDA(cudaStreamSynchronize(s));
  check_tc(ctx, u);
  SF_API_END(ctx)
}

int sf_unet_set_tensor_cores(sf_ctx* ctx, int32_t on) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && ctx->unet, SF_ERR_STATE, "no U-Net (sf_unet_init)");
  ctx->unet->use_tc = on != 0;
  SF_API_END(ctx)
}

int sf_unet_tensor_core_stats(sf_ctx* ctx, int64_t* tc_convs) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && ctx->unet, SF_ERR_STATE, "no U-Net (sf_unet_init)");
  if (tc_convs) *tc_convs = ctx->unet->tc_convs;
  SF_API_END(ctx)
}

int sf_unet_tensor_core_wait_test(sf_ctx* ctx) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null context");
  SF_CUDA(cudaSetDevice(ctx->device));
  const int flag = sf::conv3x3_tc_wait_test(ctx->stream);
  SF_REQUIRE(flag == 1, SF_ERR_STATE, "the stalled tensor-core pipeline did not report its timeout");
  SF_REQUIRE(false, SF_ERR_TIMEOUT, "tensor-core pipeline wait ran out (as the test intends); the context stays usable");
  SF_API_END(ctx)
}

// Parameters in the same flattened order (FP32 master copies); set also refreshes the
// BF16 copies.
int sf_unet_params(sf_ctx* ctx, float* get, const float* set) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && ctx->unet, SF_ERR_STATE, "no U-Net (sf_unet_init)");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfUnet* u = ctx->unet;
  int64_t off = 0;
  auto io = [&](float* d, size_t n) {
    if (get) copy_wait(get + off, d, 4 * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (set) copy_wait(d, set + off, 4 * n, cudaMemcpyHostToDevice, ctx->stream);
    off += (int64_t)n;
  };
  for (auto& c : u->convs) {
    io(c.w, c.nw);
    io(c.b, c.cout);
  }
  io(u->hw, u->base);
  io(u->hb, 1);
  if (set)
    for (auto& c : u->convs) {
      k_f32_to_bf16<<<ew_grid(ctx, c.nw), 256, 0, ctx->stream>>>((int)c.nw, c.w, c.w16);
      ctx->launches++;
    }
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  SF_API_END(ctx)
}

}  // extern "C"
