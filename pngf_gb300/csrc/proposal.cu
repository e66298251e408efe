// Learned flip proposals: a small convolutional network over the tile map.
//
// No reference counterpart. The network ranks single-tile flips by predicted
// objective change so that the exact Woodbury evaluation runs on the most
// promising tiles first; every proposal is still evaluated exactly, and a full
// exact pass is the fallback, so the network only reorders work.
//
// Input (3 channels on the tiles_y x tiles_x grid):
//   0  tile state, +-1;
//   1  Woodbury sensitivity: log of the mean |T_ee| over the tile's edges
//      (frequency 0), standardized over the map;
//   2  the tile's last exact gain (F after flip - F at that time), divided by
//      the running gain scale and clipped to [-4, 4], 0 if never evaluated.
// Network: 4 layers of 3x3 convolutions (zero padding), 3 -> C -> C -> C -> 1
// with ReLU between; weights stored in BF16 (FP32 master copy for Adam),
// activations and accumulation in FP32. Output: predicted gain / gain scale.
//
// Kernels are plain SIMT: the whole network is ~20k parameters and ~70 MFLOP
// per 41x41 map, far too small to be worth tensor-core tiles.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "pngf_internal.h"

namespace pngf {
namespace {

constexpr int NL = 4;

__global__ void k_conv_fwd(const float *__restrict__ x, const __nv_bfloat16 *__restrict__ w,
                           const float *__restrict__ bias, float *__restrict__ z, float *__restrict__ a, int Cin,
                           int Cout, int H, int W, int relu) {
  extern __shared__ float sw[];  // Cin * 9 weights of this output channel
  const int co = blockIdx.y, b = blockIdx.z;
  for (int i = threadIdx.x; i < Cin * 9; i += blockDim.x) sw[i] = __bfloat162float(w[(size_t)co * Cin * 9 + i]);
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= H * W) return;
  const int py = p / W, px = p - py * W;
  float acc = bias[co];
  const float *xb = x + (size_t)b * Cin * H * W;
  for (int ci = 0; ci < Cin; ++ci) {
    const float *xc = xb + (size_t)ci * H * W;
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      const int yy = py + ky - 1;
      if (yy < 0 || yy >= H) continue;
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const int xx = px + kx - 1;
        if (xx < 0 || xx >= W) continue;
        acc = fmaf(xc[yy * W + xx], sw[ci * 9 + ky * 3 + kx], acc);
      }
    }
  }
  const size_t o = ((size_t)b * Cout + co) * H * W + p;
  z[o] = acc;
  if (a) a[o] = relu ? fmaxf(acc, 0.f) : acc;
}

// dx[b][ci][p] = sum_co sum_k dz[b][co][p - (k - 1)] w[co][ci][k]
__global__ void k_conv_bwd_in(const float *__restrict__ dz, const __nv_bfloat16 *__restrict__ w,
                              float *__restrict__ dx, int Cin, int Cout, int H, int W) {
  extern __shared__ float sw[];  // Cout * 9 weights feeding input channel ci
  const int ci = blockIdx.y, b = blockIdx.z;
  for (int i = threadIdx.x; i < Cout * 9; i += blockDim.x) {
    const int co = i / 9, k = i - co * 9;
    sw[i] = __bfloat162float(w[((size_t)co * Cin + ci) * 9 + k]);
  }
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= H * W) return;
  const int py = p / W, px = p - py * W;
  float acc = 0.f;
  for (int co = 0; co < Cout; ++co) {
    const float *dzc = dz + ((size_t)b * Cout + co) * H * W;
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      const int yy = py - (ky - 1);
      if (yy < 0 || yy >= H) continue;
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const int xx = px - (kx - 1);
        if (xx < 0 || xx >= W) continue;
        acc = fmaf(dzc[yy * W + xx], sw[co * 9 + ky * 3 + kx], acc);
      }
    }
  }
  dx[((size_t)b * Cin + ci) * H * W + p] = acc;
}

// dw[co][ci][k] = sum_b sum_p dz[b][co][p] x[b][ci][p + k - 1]; db[co] from ci = 0.
__global__ void k_conv_bwd_w(const float *__restrict__ x, const float *__restrict__ dz, float *__restrict__ dw,
                             float *__restrict__ db, int B, int Cin, int Cout, int H, int W) {
  const int ci = blockIdx.x, co = blockIdx.y;
  float acc[10];
#pragma unroll
  for (int k = 0; k < 10; ++k) acc[k] = 0.f;
  const int HW = H * W;
  for (int idx = threadIdx.x; idx < B * HW; idx += blockDim.x) {
    const int b = idx / HW, p = idx - b * HW;
    const int py = p / W, px = p - py * W;
    const float g = dz[((size_t)b * Cout + co) * HW + p];
    const float *xc = x + ((size_t)b * Cin + ci) * HW;
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      const int yy = py + ky - 1;
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const int xx = px + kx - 1;
        if (yy >= 0 && yy < H && xx >= 0 && xx < W) acc[ky * 3 + kx] = fmaf(g, xc[yy * W + xx], acc[ky * 3 + kx]);
      }
    }
    acc[9] += g;
  }
  __shared__ float red[32][10];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 10; ++k) {
    float v = acc[k];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    float s = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i][threadIdx.x];
    if (threadIdx.x < 9) dw[((size_t)co * Cin + ci) * 9 + threadIdx.x] = s;
    else if (ci == 0) db[co] = s;
  }
}

// ---------------------------------------------------------------------------
// Tiled kernels (maps up to 64 wide, at most 32 channels, output channels a
// multiple of 8 or 1); the kernels above serve every other shape.
//
// k_conv_tile: out[b][o][p] = sum_{i,k} Wt[o][i][k] in[b][i][p + d(k)] over
// the 3x3 taps d(k) with zero padding, for one image b and a band of TH rows
// (TH = max(1, 64 / W), so at most 64 pixels). The band of the input (all
// channels, with its one-pixel halo) and the weights (transposed so that a
// thread's CO_T output channels are contiguous) sit in shared memory. The
// block's CT_KS warps split the input channels (warp w takes i = w, w + KS,
// ...); within a warp each thread accumulates CO_T channels x up to PX
// pixels, and the KS partial sums are added in a fixed order at the end.
//   forward (FLIP = false): Wt = w, out = z (+ bias), a = relu(z) if relu;
//   input gradient (FLIP = true): Wt[o][i][k] = w[i][o][8 - k] (o: an input
//   channel of the layer, i: an output channel), in = dz, out = dx, times the
//   ReLU mask (zmask > 0) of the previous layer when zmask is given.
constexpr int CT_KS = 4;
constexpr int CT_THREADS = 32 * CT_KS;
constexpr int CT_MAXC = 32;
constexpr int CT_MAXW = 64;
constexpr int CT_BAND = 64;  // target pixels per band

template <int CO_T, int PX, bool FLIP>
__global__ void __launch_bounds__(CT_THREADS) k_conv_tile(const float *__restrict__ in, const __nv_bfloat16 *__restrict__ w,
                                                          const float *__restrict__ bias, float *__restrict__ out,
                                                          float *__restrict__ a, const float *__restrict__ zmask,
                                                          int Ci, int Co, int H, int W, int TH, int relu) {
  extern __shared__ float csm[];
  const int b = blockIdx.y, y0 = blockIdx.x * TH;
  const int th = min(TH, H - y0), W2 = W + 2, plane = (TH + 2) * W2;
  const int npix = th * W;
  float *xs = csm;                        // Ci x (TH+2) x (W+2)
  float *ws = csm + (size_t)Ci * plane;   // (Ci * 9) x Co
  float *part = ws + (size_t)Ci * 9 * Co; // CT_KS x Co x npix partial sums
  for (int idx = threadIdx.x; idx < Ci * 9 * Co; idx += CT_THREADS) {
    const int o = idx % Co, ik = idx / Co, i = ik / 9, k = ik - i * 9;
    const float v = FLIP ? __bfloat162float(w[((size_t)i * Co + o) * 9 + (8 - k)])
                         : __bfloat162float(w[((size_t)o * Ci + i) * 9 + k]);
    ws[idx] = v;  // ws[(i * 9 + k) * Co + o]
  }
  const float *inb = in + (size_t)b * Ci * H * W;
  for (int idx = threadIdx.x; idx < Ci * plane; idx += CT_THREADS) {
    const int i = idx / plane, r = idx - i * plane, yy = r / W2, xx = r - yy * W2;
    const int gy = y0 + yy - 1, gx = xx - 1;
    xs[idx] = (gy >= 0 && gy < H && gx >= 0 && gx < W) ? inb[((size_t)i * H + gy) * W + gx] : 0.f;
  }
  __syncthreads();
  const int ks = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ngroups = Co / CO_T, tpg = 32 / ngroups;
  const int grp = lane / tpg, t = lane - grp * tpg;
  if (grp < ngroups) {
    int off[PX];
    bool on[PX];
#pragma unroll
    for (int j = 0; j < PX; ++j) {
      const int pp = t + j * tpg;
      on[j] = pp < npix;
      const int py = on[j] ? pp / W : 0, px = on[j] ? pp - (pp / W) * W : 0;
      off[j] = py * W2 + px;  // tap (0, 0) of pixel pp in the band
    }
    float acc[CO_T][PX];
#pragma unroll
    for (int c = 0; c < CO_T; ++c)
#pragma unroll
      for (int j = 0; j < PX; ++j) acc[c][j] = 0.f;
    for (int i = ks; i < Ci; i += CT_KS) {
      const float *xi = xs + (size_t)i * plane;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const int dk = (k / 3) * W2 + (k % 3);
        const float *wk = ws + (size_t)(i * 9 + k) * Co + grp * CO_T;
        float wv[CO_T];
#pragma unroll
        for (int c = 0; c < CO_T; ++c) wv[c] = wk[c];
#pragma unroll
        for (int j = 0; j < PX; ++j) {
          const float xv = xi[off[j] + dk];
#pragma unroll
          for (int c = 0; c < CO_T; ++c) acc[c][j] = fmaf(xv, wv[c], acc[c][j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < PX; ++j)
      if (on[j]) {
        const int pp = t + j * tpg;
#pragma unroll
        for (int c = 0; c < CO_T; ++c) part[((size_t)ks * Co + grp * CO_T + c) * npix + pp] = acc[c][j];
      }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < Co * npix; idx += CT_THREADS) {
    const int o = idx / npix, pp = idx - o * npix;
    float v = part[(size_t)o * npix + pp];
#pragma unroll
    for (int q = 1; q < CT_KS; ++q) v += part[((size_t)q * Co + o) * npix + pp];
    const size_t oi = ((size_t)b * Co + o) * H * W + (size_t)y0 * W + pp;
    if (FLIP) {
      if (zmask && zmask[oi] <= 0.f) v = 0.f;
      out[oi] = v;
    } else {
      v += bias[o];
      out[oi] = v;
      if (a) a[oi] = relu ? fmaxf(v, 0.f) : v;
    }
  }
}

// Partial weight gradients: dwp[s][o][i][k] = sum over the s-th of CT_WS
// slices of the batch of sum_p dz[b][o][p] x[b][i][p + d(k)], and the bias
// term (k = 9, sum dz) from the blocks of input channel 0. One block per
// (input channel, group of CO_T output channels, batch slice); each thread
// takes pixels p = tid, tid + 256, ..., works out which of its taps fall
// inside the map once per pixel, and walks the slice's images; a fixed-order block
// reduction, then k_conv_wsum adds the slices in order (deterministic).
constexpr int CT_WS = 4;
template <int CO_T>
__global__ void __launch_bounds__(256) k_conv_wgrad(const float *__restrict__ x, const float *__restrict__ dz,
                                                    float *__restrict__ dwp, int B, int Ci, int Co, int H, int W) {
  const int i = blockIdx.x, o0 = blockIdx.y * CO_T, sl = blockIdx.z;
  const int HW = H * W;
  const int b0 = (int)(((long)B * sl) / CT_WS), b1 = (int)(((long)B * (sl + 1)) / CT_WS);
  float acc[CO_T][10];
#pragma unroll
  for (int c = 0; c < CO_T; ++c)
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[c][k] = 0.f;
  for (int p = threadIdx.x; p < HW; p += 256) {  // this thread's pixels
    const int py = p / W, px = p - py * W;
    unsigned valid = 0;  // bit k: tap k inside the map
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int yy = py + k / 3 - 1, xx = px + k % 3 - 1;
      if (yy >= 0 && yy < H && xx >= 0 && xx < W) valid |= 1u << k;
    }
    for (int bb = b0; bb < b1; ++bb) {
      const float *xc = x + ((size_t)bb * Ci + i) * HW;
      const float *dzb = dz + ((size_t)bb * Co + o0) * HW;
      float xv[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) xv[k] = (valid >> k) & 1u ? xc[p + (k / 3 - 1) * W + (k % 3 - 1)] : 0.f;
#pragma unroll
      for (int c = 0; c < CO_T; ++c) {
        const float g = dzb[(size_t)c * HW + p];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[c][k] = fmaf(g, xv[k], acc[c][k]);
        acc[c][9] += g;
      }
    }
  }
  __shared__ float red[8][CO_T * 10];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < CO_T; ++c)
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      float v = acc[c][k];
      for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[wid][c * 10 + k] = v;
    }
  __syncthreads();
  for (int q = threadIdx.x; q < CO_T * 10; q += blockDim.x) {
    float sum = 0.f;
    for (int u = 0; u < (int)(blockDim.x >> 5); ++u) sum += red[u][q];
    const int c = q / 10, k = q - c * 10;
    dwp[(((size_t)sl * Co + o0 + c) * Ci + i) * 10 + k] = sum;
  }
}

// dw[o][i][k] = sum_s dwp[s][o][i][k], db[o] = sum_s dwp[s][o][0][9].
__global__ void k_conv_wsum(const float *__restrict__ dwp, float *__restrict__ dw, float *__restrict__ db, int Ci,
                            int Co) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = Co * Ci * 10;
  if (idx >= n) return;
  float v = 0.f;
  for (int sl = 0; sl < CT_WS; ++sl) v += dwp[(size_t)sl * n + idx];
  const int k = idx % 10, oi = idx / 10, o = oi / Ci, i = oi - o * Ci;
  if (k < 9) dw[((size_t)o * Ci + i) * 9 + k] = v;
  else if (i == 0) db[o] = v;
}

__global__ void k_relu_bwd(const float *__restrict__ z, float *__restrict__ g, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && z[i] <= 0.f) g[i] = 0.f;
}

// Masked mean squared error; out[0] += loss, dout = d loss / d y. The
// normalisation 1 / (masked entries) is inv_count, or *inv_dev when given.
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ t, const float *__restrict__ m,
                      float *__restrict__ dy, size_t n, float inv_count, const float *__restrict__ inv_dev,
                      float *loss) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (inv_dev) inv_count = *inv_dev;
  float l = 0.f;
  if (i < n) {
    const float d = (y[i] - t[i]) * m[i];
    dy[i] = 2.f * d * inv_count;
    l = d * d * inv_count;
  }
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// A training minibatch from the device sample store: for step = step[0] of
// the call, sample idx_all[step * B + b] into batch slot b (features,
// targets, masks) and 1 / (total masked entries).
__global__ void k_batch_gather(const float *__restrict__ feat, const float *__restrict__ tgt,
                               const float *__restrict__ msk, const float *__restrict__ msum,
                               const int *__restrict__ idx_all, const int *__restrict__ step, int B, int HW,
                               float *__restrict__ x, float *__restrict__ t, float *__restrict__ m,
                               float *__restrict__ inv_count) {
  const int *idx = idx_all + (size_t)step[0] * B;  // this step's minibatch
  const int b = blockIdx.y;
  const size_t i = (size_t)idx[b];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * HW; q += gridDim.x * blockDim.x)
    x[(size_t)b * 3 * HW + q] = feat[i * 3 * HW + q];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < HW; q += gridDim.x * blockDim.x) {
    t[(size_t)b * HW + q] = tgt[i * HW + q];
    m[(size_t)b * HW + q] = msk[i * HW + q];
  }
  if (b == 0 && blockIdx.x == 0 && threadIdx.x == 0) {
    float c = 0.f;  // integer-valued, exact
    for (int q = 0; q < B; ++q) c += msum[idx[q]];
    *inv_count = 1.f / fmaxf(1.f, c);
  }
}

// Adam update; the bias corrections use the step count t = step[1] + 1.
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       __nv_bfloat16 *__restrict__ wb, int n, float lr, float b1, float b2, float eps,
                       const int *__restrict__ step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float tt = (float)(step[1] + 1);
  const float c1 = 1.f - powf(b1, tt), c2 = 1.f - powf(b2, tt);
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  wb[i] = __float2bfloat16_rn(wi);
}

// End of a training step: step[0] (step of the call) and step[1] (Adam steps) advance.
__global__ void k_step_advance(int *step) {
  step[0] += 1;
  step[1] += 1;
}

__global__ void k_to_bf16(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

// Channel 1 of the features: per tile, mean log |T_ee| over its edges
// (frequency 0). One warp per tile, lanes over its edges (their diagonal
// entries load concurrently), the sum reduced in a fixed order.
template <typename TM>
__global__ void k_tile_sensitivity(const TM *__restrict__ T, long ldt, int tiles_x, int tiles_y, int cells_x,
                                   int cells_y, int ex_xsz, int ey_xsz, long nx, float *__restrict__ out) {
  const int t = (int)(((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= tiles_x * tiles_y) return;
  const int ty = t / tiles_x, tx = t - ty * tiles_x;
  const int nxe = (cells_y + 1) * cells_x, nye = cells_y * (cells_x + 1);
  double s = 0.0;
  for (int q = lane; q < nxe + nye; q += 32) {
    long e;
    if (q < nxe) {
      const int jj = q / cells_x, ii = q - jj * cells_x;
      e = (long)(tx * cells_x + ii) + (long)(ty * cells_y + jj) * ex_xsz;
    } else {
      const int r = q - nxe, jj = r / (cells_x + 1), ii = r - jj * (cells_x + 1);
      e = nx + (long)(tx * cells_x + ii) + (long)(ty * cells_y + jj) * ey_xsz;
    }
    const TM v = T[(size_t)e * ldt + e];
    s += log(hypot((double)v.x, (double)v.y) + 1e-300);
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[t] = (float)(s / (nxe + nye));
}

}  // namespace
}  // namespace pngf

using namespace pngf;

struct pngf_prop {
  Handle *h = nullptr;
  int C = 32, H = 0, W = 0, map_sz = 0;
  int cin[NL], cout[NL];
  size_t woff[NL], boff[NL], nparam = 0;
  float *d_w = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;  // fp32 params, grads, Adam moments
  __nv_bfloat16 *d_wb = nullptr;                                         // bf16 weights used by the kernels
  long adam_t = 0;
  // activations for a batch of up to cap maps
  int cap = 0;
  float *d_x = nullptr;                     // cap x 3 x H x W
  float *d_z[NL] = {}, *d_a[NL] = {};       // pre/post activations
  float *d_g1 = nullptr, *d_g2 = nullptr;   // activation gradients (cap x C x H x W)
  float *d_t = nullptr, *d_mask = nullptr;  // targets and masks (cap x H x W)
  float *d_loss = nullptr, *d_sens = nullptr, *d_inv = nullptr;
  float *d_wpart = nullptr;  // partial weight gradients of one layer (CT_WS x C x C x 10)
  // training samples (host): features and (normalized) targets / masks, and
  // per sample the number of labelled tiles
  std::vector<float> feat, tgt, msk, msum;
  long samples = 0, max_samples = 4096;
  // device copy of the sample ring (max_samples slots), up to date through
  // sample number `uploaded`; minibatch indices for one training call
  float *d_feat = nullptr, *d_tgt = nullptr, *d_msk = nullptr, *d_msum = nullptr;
  long uploaded = 0;
  int *d_idx = nullptr;
  size_t idx_cap = 0;
  // one training step as a CUDA graph (replayed per step), valid for batch
  // size graph_B and learning rate graph_lr; step counters on the device
  int *d_step = nullptr;
  cudaGraphExec_t step_exec = nullptr;
  int graph_B = 0;
  float graph_lr = 0.f;
  std::vector<float> last_gain;  // per tile, raw objective change
  double gain_scale = 0.0, gain_sq = 0.0;
  long gain_n = 0;
  // the normalized sensitivity map last computed, valid while the handle's
  // state (Handle::state_version) does not change
  std::vector<float> sens_cache;
  long sens_state = -1;
  std::mt19937 rng{1};
  std::string err;
};

namespace {

int prop_alloc_batch(pngf_prop *p, int B) {
  if (B <= p->cap) return PNGF_OK;
  if (p->step_exec) cudaGraphExecDestroy(p->step_exec);  // it refers to the buffers being replaced
  p->step_exec = nullptr;
  auto fr = [](float *&q) {
    if (q) cudaFree(q);
    q = nullptr;
  };
  fr(p->d_x);
  for (int l = 0; l < NL; ++l) {
    fr(p->d_z[l]);
    fr(p->d_a[l]);
  }
  fr(p->d_g1);
  fr(p->d_g2);
  fr(p->d_t);
  fr(p->d_mask);
  const size_t HW = (size_t)p->H * p->W;
  bool ok = cudaMalloc(&p->d_x, sizeof(float) * B * 3 * HW) == cudaSuccess;
  for (int l = 0; l < NL && ok; ++l)
    ok = cudaMalloc(&p->d_z[l], sizeof(float) * B * p->cout[l] * HW) == cudaSuccess &&
         cudaMalloc(&p->d_a[l], sizeof(float) * B * p->cout[l] * HW) == cudaSuccess;
  ok = ok && cudaMalloc(&p->d_g1, sizeof(float) * B * p->C * HW) == cudaSuccess &&
       cudaMalloc(&p->d_g2, sizeof(float) * B * p->C * HW) == cudaSuccess &&
       cudaMalloc(&p->d_t, sizeof(float) * B * HW) == cudaSuccess &&
       cudaMalloc(&p->d_mask, sizeof(float) * B * HW) == cudaSuccess;
  if (!ok) return PNGF_ERR_NOMEM;
  p->cap = B;
  return PNGF_OK;
}

// Whether the tiled kernels take this network (map width and channels).
bool tiled_ok(const pngf_prop *p) {
  return p->W <= CT_MAXW && p->C <= CT_MAXC && p->C % 8 == 0;
}

int tile_rows(const pngf_prop *p) { return std::max(1, std::min(p->H, CT_BAND / p->W)); }

size_t tile_smem(const pngf_prop *p, int ci, int co, int TH) {
  return sizeof(float) * ((size_t)ci * (TH + 2) * (p->W + 2) + (size_t)ci * 9 * co + (size_t)CT_KS * co * TH * p->W);
}

// One tiled convolution: forward (flip = false) or input gradient (flip = true).
cudaError_t conv_tile(const pngf_prop *p, bool flip, const float *in, const __nv_bfloat16 *w, const float *bias,
                      float *out, float *a, const float *zmask, int ci, int co, int B, int relu) {
  const int TH = tile_rows(p);
  const dim3 g((unsigned)((p->H + TH - 1) / TH), (unsigned)B);
  const size_t sm = tile_smem(p, ci, co, TH);
  cudaStream_t st = p->h->stream;
  cudaError_t e;
  // the shared-memory limit is raised once per kernel, to the largest band any
  // tiled shape needs (weights, input band with halo, partial sums)
  constexpr size_t kMaxSmem = sizeof(float) * ((size_t)CT_MAXC * 3 * (CT_MAXW + 2) + (size_t)CT_MAXC * 9 * CT_MAXC +
                                               (size_t)CT_KS * CT_MAXC * CT_MAXW);
  static bool raised[2][2] = {};  // [co = 1][flip]: one flag per kernel
  auto go = [&](auto kern, bool &done) {
    if (!done) {
      if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem)) !=
          cudaSuccess)
        return e;
      done = true;
    }
    if (sm > kMaxSmem) return cudaErrorInvalidValue;
    kern<<<g, CT_THREADS, sm, st>>>(in, w, bias, out, a, zmask, ci, co, p->H, p->W, TH, relu);
    return cudaGetLastError();
  };
  // a band has at most CT_MAXW pixels; a warp's 32 / (co / 8) threads of one
  // group of 8 channels take at most 8 pixels each (co = 1: 32 threads, 2)
  static_assert(CT_MAXW <= 8 * (32 / (CT_MAXC / 8)) && CT_BAND <= CT_MAXW, "pixels per thread");
  if (co % 8 == 0)
    return flip ? go(k_conv_tile<8, 8, true>, raised[0][1]) : go(k_conv_tile<8, 8, false>, raised[0][0]);
  return flip ? go(k_conv_tile<1, 2, true>, raised[1][1]) : go(k_conv_tile<1, 2, false>, raised[1][0]);  // co = 1
}

// Weight and bias gradients of layer l (tiled path).
cudaError_t conv_wgrad(pngf_prop *p, int l, const float *xin, const float *dz, int B) {
  cudaStream_t st = p->h->stream;
  const int ci = p->cin[l], co = p->cout[l];
  if (co % 8 == 0)
    k_conv_wgrad<8><<<dim3(ci, co / 8, CT_WS), 256, 0, st>>>(xin, dz, p->d_wpart, B, ci, co, p->H, p->W);
  else
    k_conv_wgrad<1><<<dim3(ci, co, CT_WS), 256, 0, st>>>(xin, dz, p->d_wpart, B, ci, co, p->H, p->W);
  const int n = co * ci * 10;
  k_conv_wsum<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p->d_wpart, p->d_g + p->woff[l], p->d_g + p->boff[l], ci,
                                                            co);
  return cudaGetLastError();
}

cudaError_t prop_forward(pngf_prop *p, int B) {
  const int HW = p->H * p->W;
  const float *in = p->d_x;
  for (int l = 0; l < NL; ++l) {
    if (tiled_ok(p)) {
      const cudaError_t e = conv_tile(p, false, in, p->d_wb + p->woff[l], p->d_w + p->boff[l], p->d_z[l], p->d_a[l],
                                      nullptr, p->cin[l], p->cout[l], B, l < NL - 1 ? 1 : 0);
      if (e != cudaSuccess) return e;
    } else {
      dim3 g((HW + 127) / 128, p->cout[l], B);
      k_conv_fwd<<<g, 128, sizeof(float) * p->cin[l] * 9, p->h->stream>>>(
          in, p->d_wb + p->woff[l], p->d_w + p->boff[l], p->d_z[l], p->d_a[l], p->cin[l], p->cout[l], p->H, p->W,
          l < NL - 1 ? 1 : 0);
    }
    in = p->d_a[l];
  }
  return cudaGetLastError();
}

// Backward from d(output) in d_g1 (B x 1 x H x W); fills d_g.
cudaError_t prop_backward(pngf_prop *p, int B) {
  const int HW = p->H * p->W;
  float *gcur = p->d_g1, *gnext = p->d_g2;
  if (tiled_ok(p)) {
    // the ReLU mask of layer l - 1 is applied as layer l's input gradient is written
    for (int l = NL - 1; l >= 0; --l) {
      const float *xin = l == 0 ? p->d_x : p->d_a[l - 1];
      const cudaError_t ew = conv_wgrad(p, l, xin, gcur, B);
      if (ew != cudaSuccess) return ew;
      if (l > 0) {
        const cudaError_t e = conv_tile(p, true, gcur, p->d_wb + p->woff[l], nullptr, gnext, nullptr, p->d_z[l - 1],
                                        p->cout[l], p->cin[l], B, 0);
        if (e != cudaSuccess) return e;
        std::swap(gcur, gnext);
      }
    }
    return cudaGetLastError();
  }
  for (int l = NL - 1; l >= 0; --l) {
    if (l < NL - 1) {
      const size_t n = (size_t)B * p->cout[l] * HW;
      k_relu_bwd<<<(unsigned)((n + 255) / 256), 256, 0, p->h->stream>>>(p->d_z[l], gcur, n);
    }
    const float *xin = l == 0 ? p->d_x : p->d_a[l - 1];
    k_conv_bwd_w<<<dim3(p->cin[l], p->cout[l]), 256, 0, p->h->stream>>>(xin, gcur, p->d_g + p->woff[l],
                                                                        p->d_g + p->boff[l], B, p->cin[l],
                                                                        p->cout[l], p->H, p->W);
    if (l > 0) {
      dim3 g((HW + 127) / 128, p->cin[l], B);
      k_conv_bwd_in<<<g, 128, sizeof(float) * p->cout[l] * 9, p->h->stream>>>(gcur, p->d_wb + p->woff[l], gnext,
                                                                               p->cin[l], p->cout[l], p->H, p->W);
      std::swap(gcur, gnext);
    }
  }
  return cudaGetLastError();
}

int prop_err(pngf_prop *p, int code, const std::string &m) {
  p->err = m;
  return code;
}

bool eligible(const Handle *h, int t) {
  const int xsz = h->cfg.tiles_x, ysz = h->cfg.tiles_y;
  const int mx = (int)((xsz - 1) * 0.5), my = (int)((ysz - 1) * 0.5);
  const int ty = t / xsz, tx = t - ty * xsz;
  if (ty == my && (tx == mx || tx == mx - 1 || tx == mx + 1)) return false;
  return true;
}

// Brings the device copy of the sample ring up to date with the host ring
// (the slots written since the last upload, as at most two contiguous runs).
int prop_upload_samples(pngf_prop *p) {
  const size_t HW = (size_t)p->map_sz, cap = (size_t)p->max_samples;
  cudaStream_t s = p->h->stream;
  if (!p->d_feat) {
    if (cudaMalloc(&p->d_feat, sizeof(float) * cap * 3 * HW) != cudaSuccess ||
        cudaMalloc(&p->d_tgt, sizeof(float) * cap * HW) != cudaSuccess ||
        cudaMalloc(&p->d_msk, sizeof(float) * cap * HW) != cudaSuccess ||
        cudaMalloc(&p->d_msum, sizeof(float) * cap) != cudaSuccess)
      return prop_err(p, PNGF_ERR_NOMEM, "sample store");
  }
  long from = std::max(p->uploaded, p->samples - p->max_samples);
  while (from < p->samples) {
    const size_t slot = (size_t)(from % p->max_samples);
    const size_t cnt = std::min((size_t)(p->samples - from), cap - slot);
    bool ok = cudaMemcpyAsync(p->d_feat + slot * 3 * HW, &p->feat[slot * 3 * HW], sizeof(float) * cnt * 3 * HW,
                              cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(p->d_tgt + slot * HW, &p->tgt[slot * HW], sizeof(float) * cnt * HW,
                              cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(p->d_msk + slot * HW, &p->msk[slot * HW], sizeof(float) * cnt * HW,
                              cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(p->d_msum + slot, &p->msum[slot], sizeof(float) * cnt, cudaMemcpyHostToDevice, s) ==
                  cudaSuccess;
    if (!ok) return prop_err(p, PNGF_ERR_CUDA, "sample upload");
    from += (long)cnt;
  }
  p->uploaded = p->samples;
  return PNGF_OK;
}

// One training step on the minibatch of step d_step[0]: gather, forward,
// masked MSE, backward, Adam, counters advanced. Enqueue-only (capturable).
cudaError_t train_step(pngf_prop *p, int batch, float lr) {
  cudaStream_t s = p->h->stream;
  const int HW = p->map_sz;
  const size_t n = (size_t)batch * HW;
  k_batch_gather<<<dim3((unsigned)((3 * HW + 255) / 256), (unsigned)batch), 256, 0, s>>>(
      p->d_feat, p->d_tgt, p->d_msk, p->d_msum, p->d_idx, p->d_step, batch, HW, p->d_x, p->d_t, p->d_mask, p->d_inv);
  cudaError_t e = prop_forward(p, batch);
  if (e != cudaSuccess) return e;
  k_mse<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p->d_z[NL - 1], p->d_t, p->d_mask, p->d_g1, n, 1.f, p->d_inv,
                                                     p->d_loss);
  if ((e = prop_backward(p, batch)) != cudaSuccess) return e;
  k_adam<<<(unsigned)((p->nparam + 255) / 256), 256, 0, s>>>(p->d_w, p->d_g, p->d_m, p->d_v, p->d_wb, (int)p->nparam,
                                                             lr, 0.9f, 0.999f, 1e-8f, p->d_step);
  k_step_advance<<<1, 1, 0, s>>>(p->d_step);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int pngf_prop_create(pngf_handle *ph, int channels, unsigned long long seed, pngf_prop **out) {
  Handle *h = reinterpret_cast<Handle *>(ph);
  if (!h || !out || channels < 1 || channels > 128) return PNGF_ERR_ARG;
  pngf_prop *p = new pngf_prop();
  p->h = h;
  p->C = channels;
  p->H = h->cfg.tiles_y;
  p->W = h->cfg.tiles_x;
  p->map_sz = h->map_sz;
  p->rng.seed((unsigned)seed);
  const int cin[NL] = {3, channels, channels, channels}, cout[NL] = {channels, channels, channels, 1};
  size_t off = 0;
  for (int l = 0; l < NL; ++l) {
    p->cin[l] = cin[l];
    p->cout[l] = cout[l];
    p->woff[l] = off;
    off += (size_t)cout[l] * cin[l] * 9;
    p->boff[l] = off;
    off += cout[l];
  }
  p->nparam = off;
  // He-normal initialisation, zero biases
  std::vector<float> w(off, 0.f);
  for (int l = 0; l < NL; ++l) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (cin[l] * 9)));
    for (size_t i = 0; i < (size_t)cout[l] * cin[l] * 9; ++i) w[p->woff[l] + i] = nd(p->rng);
  }
  bool ok = cudaMalloc(&p->d_w, sizeof(float) * off) == cudaSuccess &&
            cudaMalloc(&p->d_g, sizeof(float) * off) == cudaSuccess &&
            cudaMalloc(&p->d_m, sizeof(float) * off) == cudaSuccess &&
            cudaMalloc(&p->d_v, sizeof(float) * off) == cudaSuccess &&
            cudaMalloc(&p->d_wb, sizeof(__nv_bfloat16) * off) == cudaSuccess &&
            cudaMalloc(&p->d_loss, sizeof(float)) == cudaSuccess &&
            cudaMalloc(&p->d_inv, sizeof(float)) == cudaSuccess &&
            cudaMalloc(&p->d_step, 2 * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&p->d_wpart, sizeof(float) * CT_WS * channels * std::max(channels, 3) * 10) == cudaSuccess &&
            cudaMalloc(&p->d_sens, sizeof(float) * p->map_sz) == cudaSuccess;
  if (!ok || prop_alloc_batch(p, 64) != PNGF_OK) {
    pngf_prop_destroy(p);
    return PNGF_ERR_NOMEM;
  }
  cudaMemcpy(p->d_w, w.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  cudaMemset(p->d_m, 0, sizeof(float) * off);
  cudaMemset(p->d_v, 0, sizeof(float) * off);
  k_to_bf16<<<(unsigned)((off + 255) / 256), 256>>>(p->d_w, p->d_wb, (int)off);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    pngf_prop_destroy(p);
    return PNGF_ERR_CUDA;
  }
  p->last_gain.assign(p->map_sz, 0.f);
  *out = p;
  return PNGF_OK;
}

int pngf_prop_destroy(pngf_prop *p) {
  if (!p) return PNGF_OK;
  auto fr = [](void *q) {
    if (q) cudaFree(q);
  };
  fr(p->d_w);
  fr(p->d_g);
  fr(p->d_m);
  fr(p->d_v);
  fr(p->d_wb);
  fr(p->d_loss);
  fr(p->d_inv);
  fr(p->d_wpart);
  fr(p->d_feat);
  fr(p->d_tgt);
  fr(p->d_msk);
  fr(p->d_msum);
  fr(p->d_idx);
  fr(p->d_step);
  if (p->step_exec) cudaGraphExecDestroy(p->step_exec);
  fr(p->d_sens);
  fr(p->d_x);
  for (int l = 0; l < NL; ++l) {
    fr(p->d_z[l]);
    fr(p->d_a[l]);
  }
  fr(p->d_g1);
  fr(p->d_g2);
  fr(p->d_t);
  fr(p->d_mask);
  delete p;
  return PNGF_OK;
}

long pngf_prop_num_params(const pngf_prop *p) { return p ? (long)p->nparam : 0; }

int pngf_prop_get_params(const pngf_prop *p, float *w) {
  if (!p || !w) return PNGF_ERR_ARG;
  return cudaMemcpy(w, p->d_w, sizeof(float) * p->nparam, cudaMemcpyDeviceToHost) == cudaSuccess ? PNGF_OK
                                                                                                 : PNGF_ERR_CUDA;
}

int pngf_prop_set_params(pngf_prop *p, const float *w) {
  if (!p || !w) return PNGF_ERR_ARG;
  if (cudaMemcpy(p->d_w, w, sizeof(float) * p->nparam, cudaMemcpyHostToDevice) != cudaSuccess) return PNGF_ERR_CUDA;
  k_to_bf16<<<(unsigned)((p->nparam + 255) / 256), 256, 0, p->h->stream>>>(p->d_w, p->d_wb, (int)p->nparam);
  return cudaStreamSynchronize(p->h->stream) == cudaSuccess ? PNGF_OK : PNGF_ERR_CUDA;
}

// Forward and backward on caller-given inputs (B x 3 x H x W), targets and
// masks (B x H x W): output (B x H x W), loss and gradients (nparam), all host
// memory. For gradient checks.
int pngf_prop_forward_backward(pngf_prop *p, const float *x, int B, const float *target, const float *mask,
                               float *out, float *grad, float *loss) {
  if (!p || !x || B < 1) return PNGF_ERR_ARG;
  int rc = prop_alloc_batch(p, B);
  if (rc) return rc;
  cudaStream_t s = p->h->stream;
  const size_t HW = (size_t)p->H * p->W;
  cudaMemcpyAsync(p->d_x, x, sizeof(float) * B * 3 * HW, cudaMemcpyHostToDevice, s);
  if (prop_forward(p, B) != cudaSuccess) return PNGF_ERR_CUDA;
  if (out) cudaMemcpyAsync(out, p->d_z[NL - 1], sizeof(float) * B * HW, cudaMemcpyDeviceToHost, s);
  if (target && mask) {
    cudaMemcpyAsync(p->d_t, target, sizeof(float) * B * HW, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(p->d_mask, mask, sizeof(float) * B * HW, cudaMemcpyHostToDevice, s);
    double msum = 0.0;
    for (size_t i = 0; i < B * HW; ++i) msum += mask[i];
    cudaMemsetAsync(p->d_loss, 0, sizeof(float), s);
    const size_t n = B * HW;
    k_mse<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p->d_z[NL - 1], p->d_t, p->d_mask, p->d_g1, n,
                                                       (float)(1.0 / std::max(1.0, msum)), nullptr, p->d_loss);
    if (prop_backward(p, B) != cudaSuccess) return PNGF_ERR_CUDA;
    if (grad) cudaMemcpyAsync(grad, p->d_g, sizeof(float) * p->nparam, cudaMemcpyDeviceToHost, s);
    if (loss) cudaMemcpyAsync(loss, p->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  }
  return cudaStreamSynchronize(s) == cudaSuccess ? PNGF_OK : PNGF_ERR_CUDA;
}

// Features of the handle's current design (3 x H x W), written to the device
// input slot `slot` and, if feat is not NULL, to host memory.
static int prop_features(pngf_prop *p, int slot, float *feat) {
  Handle *h = p->h;
  if (!h->prepared) return prop_err(p, PNGF_ERR_STATE, "handle not prepared");
  const int HW = p->map_sz;
  if (p->sens_state != h->state_version || (int)p->sens_cache.size() != HW) {  // the sensitivity map
    if (h->cfg.precision == PNGF_PREC_FP64)
      k_tile_sensitivity<double2><<<(HW + 3) / 4, 128, 0, h->stream>>>(
          h->f[0].M64, h->ldm, h->cfg.tiles_x, h->cfg.tiles_y, h->cfg.cells_x, h->cfg.cells_y, h->ex_xsz, h->ey_xsz,
          h->nx, p->d_sens);
    else
      k_tile_sensitivity<float2><<<(HW + 3) / 4, 128, 0, h->stream>>>(
          h->f[0].T32, h->ldm, h->cfg.tiles_x, h->cfg.tiles_y, h->cfg.cells_x, h->cfg.cells_y, h->ex_xsz, h->ey_xsz,
          h->nx, p->d_sens);
    std::vector<float> sens(HW);
    if (cudaMemcpyAsync(sens.data(), p->d_sens, sizeof(float) * HW, cudaMemcpyDeviceToHost, h->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
      return prop_err(p, PNGF_ERR_CUDA, "feature extraction");
    double mu = 0.0, sd = 0.0;
    for (float v : sens) mu += v;
    mu /= HW;
    for (float v : sens) sd += (v - mu) * (v - mu);
    sd = std::sqrt(sd / HW) + 1e-12;
    p->sens_cache.resize(HW);
    for (int t = 0; t < HW; ++t) p->sens_cache[t] = (float)((sens[t] - mu) / sd);
    p->sens_state = h->state_version;
  }
  std::vector<float> f(3 * HW);
  const double gs = p->gain_scale > 0 ? p->gain_scale : 1.0;
  for (int t = 0; t < HW; ++t) {
    f[t] = h->tile_map[t] ? 1.f : -1.f;
    f[HW + t] = p->sens_cache[t];
    f[2 * HW + t] = (float)std::max(-4.0, std::min(4.0, p->last_gain[t] / gs));
  }
  if (feat) std::memcpy(feat, f.data(), sizeof(float) * 3 * HW);
  if (slot >= 0 &&
      cudaMemcpyAsync(p->d_x + (size_t)slot * 3 * HW, f.data(), sizeof(float) * 3 * HW, cudaMemcpyHostToDevice,
                      h->stream) != cudaSuccess)
    return prop_err(p, PNGF_ERR_CUDA, "feature upload");
  return PNGF_OK;
}

int pngf_prop_features(pngf_prop *p, float *feat) {
  if (!p) return PNGF_ERR_ARG;
  return prop_features(p, -1, feat);
}

// Records exact gains (F after flip - F now) of single-tile flips at the
// handle's current design: updates each tile's last gain and stores one
// training sample (features, normalized gains, mask).
int pngf_prop_record(pngf_prop *p, const int *tiles, const double *gains, int count) {
  if (!p || (count > 0 && (!tiles || !gains))) return PNGF_ERR_ARG;
  const int HW = p->map_sz;
  std::vector<float> f(3 * HW);
  int rc = prop_features(p, -1, f.data());
  if (rc) return rc;
  for (int i = 0; i < count; ++i) {
    if (tiles[i] < 0 || tiles[i] >= HW) return prop_err(p, PNGF_ERR_ARG, "tile index out of range");
    if (!std::isfinite(gains[i])) continue;  // singular capacitance: no label
    p->gain_sq += gains[i] * gains[i];
    ++p->gain_n;
  }
  if (p->gain_n > 0) p->gain_scale = std::sqrt(p->gain_sq / p->gain_n);
  std::vector<float> t(HW, 0.f), m(HW, 0.f);
  const double gs = p->gain_scale > 0 ? p->gain_scale : 1.0;
  for (int i = 0; i < count; ++i) {
    if (!std::isfinite(gains[i])) continue;
    const int tile = tiles[i];
    t[tile] = (float)std::max(-8.0, std::min(8.0, gains[i] / gs));
    m[tile] = 1.f;
  }
  // Ring buffer of samples.
  const long slot = p->samples % p->max_samples;
  if ((long)p->feat.size() < (slot + 1) * 3 * HW) {
    p->feat.resize((slot + 1) * 3 * HW);
    p->tgt.resize((slot + 1) * HW);
    p->msk.resize((slot + 1) * HW);
    p->msum.resize(slot + 1);
  }
  std::memcpy(&p->feat[slot * 3 * HW], f.data(), sizeof(float) * 3 * HW);
  std::memcpy(&p->tgt[slot * HW], t.data(), sizeof(float) * HW);
  std::memcpy(&p->msk[slot * HW], m.data(), sizeof(float) * HW);
  float labelled = 0.f;
  for (float v : m) labelled += v;
  p->msum[slot] = labelled;
  ++p->samples;
  for (int i = 0; i < count; ++i)
    if (std::isfinite(gains[i])) p->last_gain[tiles[i]] = (float)gains[i];
  return PNGF_OK;
}

long pngf_prop_num_samples(const pngf_prop *p) { return p ? std::min(p->samples, p->max_samples) : 0; }

// Adam steps on random minibatches of the stored samples; *loss = mean loss.
int pngf_prop_train(pngf_prop *p, int steps, int batch, float lr, float *loss) {
  pngf::TraceRange trace_("pngf_prop_train");
  if (!p || steps < 0 || batch < 1) return PNGF_ERR_ARG;
  const long have = std::min(p->samples, p->max_samples);
  if (have == 0) return prop_err(p, PNGF_ERR_STATE, "no training samples");
  int rc = prop_alloc_batch(p, batch);
  if (rc) return rc;
  cudaStream_t s = p->h->stream;
  rc = prop_upload_samples(p);
  if (rc) return rc;
  // every minibatch of this call drawn up front (the same draws, in the same
  // order, as one at a time), then the steps run back to back on the device
  // with no host round trip; the loss is read once at the end
  std::uniform_int_distribution<long> pick(0, have - 1);
  std::vector<int> idx((size_t)steps * batch);
  for (auto &v : idx) v = (int)pick(p->rng);
  if (idx.size() > p->idx_cap) {
    if (p->step_exec) cudaGraphExecDestroy(p->step_exec);  // it refers to d_idx
    p->step_exec = nullptr;
    if (p->d_idx) cudaFree(p->d_idx);
    p->d_idx = nullptr;
    p->idx_cap = 0;
    if (cudaMalloc(&p->d_idx, sizeof(int) * idx.size()) != cudaSuccess) return prop_err(p, PNGF_ERR_NOMEM, "indices");
    p->idx_cap = idx.size();
  }
  if (steps > 0 &&
      cudaMemcpyAsync(p->d_idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return prop_err(p, PNGF_ERR_CUDA, "index upload");
  cudaMemsetAsync(p->d_loss, 0, sizeof(float), s);
  const int step0[2] = {0, (int)p->adam_t};
  if (cudaMemcpyAsync(p->d_step, step0, sizeof(step0), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return prop_err(p, PNGF_ERR_CUDA, "step counters");
  // the first step runs eagerly (it also raises the kernels' shared-memory
  // limits); the others replay a captured graph of one step
  for (int it = 0; it < steps; ++it) {
    if (it > 0 && p->step_exec && p->graph_B == batch && p->graph_lr == lr) {
      if (cudaGraphLaunch(p->step_exec, s) != cudaSuccess) return prop_err(p, PNGF_ERR_CUDA, "training step graph");
      continue;
    }
    if (it > 0) {
      if (p->step_exec) cudaGraphExecDestroy(p->step_exec);
      p->step_exec = nullptr;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return prop_err(p, PNGF_ERR_CUDA, "training step capture");
      const cudaError_t ec = train_step(p, batch, lr);
      const cudaError_t ee = cudaStreamEndCapture(s, &g);
      if (ec != cudaSuccess || ee != cudaSuccess || cudaGraphInstantiate(&p->step_exec, g, 0) != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        p->step_exec = nullptr;
        return prop_err(p, PNGF_ERR_CUDA, "training step capture");
      }
      cudaGraphDestroy(g);
      p->graph_B = batch;
      p->graph_lr = lr;
      if (cudaGraphLaunch(p->step_exec, s) != cudaSuccess) return prop_err(p, PNGF_ERR_CUDA, "training step graph");
      continue;
    }
    if (train_step(p, batch, lr) != cudaSuccess) return prop_err(p, PNGF_ERR_CUDA, "training step");
  }
  p->adam_t += steps;
  float l = 0.f;
  if (cudaMemcpyAsync(&l, p->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return prop_err(p, PNGF_ERR_CUDA, "training steps");
  if (loss) *loss = steps > 0 ? l / (float)steps : 0.f;
  return PNGF_OK;
}

// Predicted gain (in units of the gain scale) of flipping each tile of the
// handle's current design; tiles that are never candidates get +inf.
int pngf_prop_predict(pngf_prop *p, float *pred) {
  if (!p || !pred) return PNGF_ERR_ARG;
  int rc = prop_features(p, 0, nullptr);
  if (rc) return rc;
  if (prop_forward(p, 1) != cudaSuccess) return prop_err(p, PNGF_ERR_CUDA, "forward");
  if (cudaMemcpyAsync(pred, p->d_z[NL - 1], sizeof(float) * p->map_sz, cudaMemcpyDeviceToHost, p->h->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(p->h->stream) != cudaSuccess)
    return prop_err(p, PNGF_ERR_CUDA, "prediction");
  for (int t = 0; t < p->map_sz; ++t)
    if (!eligible(p->h, t)) pred[t] = INFINITY;
  return PNGF_OK;
}

const char *pngf_prop_last_error(const pngf_prop *p) { return p ? p->err.c_str() : "null"; }

}  // extern "C"
