// FP64 kernels of the PNGF hot path on sm_103a.
//
// Layout in HBM, per frequency: M = [[T, y], [R, Eobj]] row-major,
// (N+E) rows x ldm columns (ldm >= N+1, padded to a multiple of 16 elements);
// Einc (N); G (N x N column-major, as loaded). P (int8, N) and the tile map
// are shared by all frequencies.
//
// Kernels:
//   k_init_M        M for P = 0 (T = G - I, R = Gobj, y = 0, Eobj = 0), Einc
//                   and the port constants (pngfopt.hpp:559-618).
//   k_edge_lists    flipped-edge list of each candidate: the edges whose P
//                   changes, ascending, with signs (pngfopt.hpp:384-418).
//   k_eval          one CTA per (candidate, frequency): gathers T[s,s], y_s,
//                   R[:,s], forms K = I + T[s,s] D, LU with partial pivoting
//                   in shared memory, solves, forms newEobj and the objective
//                   term (pngfopt.hpp:379-539 and main.cpp:406-416).
//   k_score         F = sum over frequencies, first candidate with F < F_best
//                   (main.cpp:418-429).
//   k_acc_factor    accept step: K, its LU and z = D (Einc_s + K^-1 w).
//   k_acc_W         W = [D K^-1 M[s, 0:N], z] (k x (N+1)).
//   k_acc_gather    A = M[:, s] ((N+E) x k, column-major).
//   k_rank_update   M -= A W (replaces update_C_inv's zgemm, pngfopt.hpp:350-358,
//                   and compute_R_matrix(0)).
#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>
#include <vector>

#include "bounds.cuh"
#include "pngf_internal.h"

namespace pngf {

// Complex arithmetic with every fused multiply-add written out, so that the
// rounding does not depend on how the compiler contracts an expression in a
// given kernel: the CTA- and warp-per-candidate evaluation kernels (and the
// accept prologue) then produce bit-identical results.
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(__fma_rn(a.x, b.x, __dmul_rn(-a.y, b.y)), __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x)));
}
// a - b*c
__device__ __forceinline__ double2 cfnma(double2 a, double2 b, double2 c) {
  return make_double2(__fma_rn(b.y, c.y, __fma_rn(-b.x, c.x, a.x)), __fma_rn(-b.y, c.x, __fma_rn(-b.x, c.y, a.y)));
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }
// Pivot key of a complex entry: the bit pattern of |re| + |im| (LAPACK's
// izamax measure) as an integer -- non-negative doubles order like their bit
// patterns, so the argmax over a column runs on the integer pipes and only
// the one add uses GB300's narrow FP64 pipe. A NaN measure gets -1, so that,
// as with a floating-point compare, it is never chosen.
__device__ __forceinline__ long long pivot_key(double2 a) {
  const long long b = __double_as_longlong(cabs1(a));
  return (b & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll ? -1ll : b;
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double den = __fma_rn(b.x, b.x, __dmul_rn(b.y, b.y));
  return make_double2(__ddiv_rn(__fma_rn(a.x, b.x, __dmul_rn(a.y, b.y)), den),
                      __ddiv_rn(__fma_rn(a.y, b.x, __dmul_rn(-a.x, b.y)), den));
}
// 1 / p, as the LU's column scaling uses it.
__device__ __forceinline__ double2 crecip(double2 p) {
  const double den = __fma_rn(p.x, p.x, __dmul_rn(p.y, p.y));
  return make_double2(__ddiv_rn(p.x, den), __ddiv_rn(-p.y, den));
}
__device__ __forceinline__ double2 shfl2(double2 v, int src) {
  return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

template <typename T> __device__ __forceinline__ double2 ldM(const T *M, size_t i);
template <> __device__ __forceinline__ double2 ldM<double2>(const double2 *M, size_t i) { return M[i]; }
template <> __device__ __forceinline__ double2 ldM<float2>(const float2 *M, size_t i) {
  const float2 v = M[i];
  return make_double2(v.x, v.y);
}

// Read-only view of one frequency's state: the T block (N x N, leading
// dimension ldt, FP64 or complex64), the y column (y_i = y[i*ys]) and the E
// objective rows (R[e*ldr + j], with Eobj_e at column N). In the FP64 layout
// all three live in M; in the complex64 layout T is stored in complex64 and y,
// R, Eobj stay in FP64.
//
// Deferred updates (complex64 layout, rp > 0): the stored T lags the true T
// by the pending rank-rp correction, T_true = T - U Vt^T with U and Vt N x rp
// complex64 (row i of each at [i * rcap]); t() returns T_true, the correction
// summed in FP32.
template <typename TM> struct SV {
  const TM *T;
  long ldt;
  const double2 *y;
  long ys;
  const double2 *R;
  long ldr;
  const float2 *U = nullptr;
  const float2 *Vt = nullptr;
  int rp = 0;
  int rcap = 0;
  long bn = 0;  // bounds-checked build: N, the extent every edge index must fall in (0 = unchecked)
  int be = 0;   // ... and E, the objective rows
  __device__ __forceinline__ double2 t(size_t i, size_t j) const {
    if (bn && !PNGF_BOUNDS_OK(i < (size_t)bn && j < (size_t)bn, kBoundsT, (long long)i, (long long)j))
      return make_double2(0.0, 0.0);
    double2 v = ldM(T, i * ldt + j);
    if (rp > 0) {
      const float2 *u = U + i * rcap, *w = Vt + j * rcap;
      float cx = 0.f, cy = 0.f;
      for (int q = 0; q < rp; ++q) {
        const float2 a = u[q], b = w[q];
        cx = fmaf(a.x, b.x, fmaf(-a.y, b.y, cx));
        cy = fmaf(a.x, b.y, fmaf(a.y, b.x, cy));
      }
      v.x -= (double)cx;
      v.y -= (double)cy;
    }
    return v;
  }
  __device__ __forceinline__ double2 yv(size_t i) const {
    if (bn && !PNGF_BOUNDS_OK(i < (size_t)bn, kBoundsY, (long long)i, 0)) return make_double2(0.0, 0.0);
    return y[i * ys];
  }
  __device__ __forceinline__ double2 r(int e, size_t j) const {
    if (bn && !PNGF_BOUNDS_OK(e >= 0 && e < be && j <= (size_t)bn, kBoundsR, e, (long long)j))
      return make_double2(0.0, 0.0);
    return R[(size_t)e * ldr + j];
  }
};

// Einc[e] for an edge index from an edge list.
__device__ __forceinline__ double2 einc_at(const double2 *__restrict__ Einc, long e, long n) {
  if (!PNGF_BOUNDS_OK(e >= 0 && e < n, kBoundsEinc, e, 0)) return make_double2(0.0, 0.0);
  return Einc[e];
}

struct Geo {
  int tiles_x, tiles_y, cells_x, cells_y;
  int ex_xsz, ey_xsz;
  long nx;
  int map_sz;
  int max_flips;
  int kmax;
};

struct ObjConst {
  double dx, dy, dz;
};

__host__ Geo make_geo(const Handle *h) {
  Geo g;
  g.tiles_x = h->cfg.tiles_x;
  g.tiles_y = h->cfg.tiles_y;
  g.cells_x = h->cfg.cells_x;
  g.cells_y = h->cfg.cells_y;
  g.ex_xsz = h->ex_xsz;
  g.ey_xsz = h->ey_xsz;
  g.nx = h->nx;
  g.map_sz = h->map_sz;
  g.max_flips = h->cfg.max_flips;
  g.kmax = h->kmax;
  return g;
}

// One frequency's objective term (main.cpp:407-413). perf = (Re S11, Im S11, D).
// Not inlined, so every kernel that calls it rounds it the same way.
__device__ __noinline__ double objective_term(const double2 *eo, int E, const FreqConst &fc, const ObjConst &oc,
                                 double *perf) {
  const double2 v = cadd(eo[0], fc.vinc);
  double2 zin = make_double2(-v.x * oc.dx * 0.5 / (2.0 * oc.dy * oc.dz),
                             -v.y * oc.dx * 0.5 / (2.0 * oc.dy * oc.dz));
  const double2 s11 = cdiv(make_double2(zin.x - 50.0, zin.y), make_double2(zin.x + 50.0, zin.y));
  double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
  if (E > 1) a = cadd(eo[1], fc.ln1);
  if (E > 2) b = cadd(eo[2], fc.ln2);
  const double eta0 = 3.767303134118051e+02;
  double D = (fc.k0 * fc.k0 / (32.0 * M_PI * M_PI * eta0)) * (a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y);
  const double pin = -v.x * oc.dx * 0.5 * (2.0 * oc.dy * oc.dz) * 0.5;
  D = 4.0 * M_PI * D / pin;
  const double m = hypot(s11.x, s11.y);
  perf[0] = s11.x;
  perf[1] = s11.y;
  perf[2] = D;
  return 200.0 * m * m + (15.0 - D) * (15.0 - D);
}

// ---------------------------------------------------------------------------
// init

__global__ void k_init_M_tile(const double2 *__restrict__ G, long n, long ldm, double2 *__restrict__ M) {
  // 32x32 tile transpose: M[i][j] = G(i, j) - delta_ij, G column-major.
  __shared__ double2 tile[32][33];
  const long j0 = (long)blockIdx.x * 32, i0 = (long)blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const long j = j0 + r, i = i0 + tx;
    tile[r][tx] = (i < n && j < n) ? G[(size_t)j * n + i] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const long i = i0 + r, j = j0 + tx;
    if (i < n && j < ldm) {
      double2 v = (j < n) ? tile[tx][r] : make_double2(0.0, 0.0);
      if (i == j) v.x -= 1.0;
      M[(size_t)i * ldm + j] = v;
    }
  }
}

// Objective rows of M (rows N..N+E-1), Einc, and column N zeroed.
__global__ void k_init_M_rows(const double2 *__restrict__ G, const double2 *__restrict__ gobj, long n, int E,
                              long ldm, const long *__restrict__ port, int nport, double2 *__restrict__ M,
                              double2 *__restrict__ Einc) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ldm) return;
  if (j < n) {
    double2 g0 = make_double2(0.0, 0.0), e = make_double2(0.0, 0.0);
    for (int p = 0; p < nport; ++p) {
      g0 = cadd(g0, G[(size_t)j * n + port[p]]);  // row p of G: Gobj row 0 (pngfopt.hpp:592)
      e = cadd(e, G[(size_t)port[p] * n + j]);    // column p of G: Einc (pngfopt.hpp:594)
    }
    M[(size_t)n * ldm + j] = g0;
    Einc[j] = e;
    for (int r = 1; r < E; ++r) M[(size_t)(n + r) * ldm + j] = gobj[(size_t)(r - 1) * n + j];
  } else {
    for (int r = 0; r < E; ++r) M[(size_t)(n + r) * ldm + j] = make_double2(0.0, 0.0);
  }
  if (j < n + E) M[(size_t)j * ldm + n] = make_double2(0.0, 0.0);  // y = 0, Eobj = 0 for P = 0
}

__global__ void k_port_const(const double2 *__restrict__ Einc, const double2 *__restrict__ gobj, long n, int E,
                             const long *__restrict__ port, int nport, double k0, FreqConst *out) {
  FreqConst c;
  c.vinc = c.ln1 = c.ln2 = make_double2(0.0, 0.0);
  for (int p = 0; p < nport; ++p) {
    if (E > 1) c.ln1 = cadd(c.ln1, gobj[port[p]]);
    if (E > 2) c.ln2 = cadd(c.ln2, gobj[(size_t)n + port[p]]);
  }
  for (int p = 0; p < nport; ++p) c.vinc = cadd(c.vinc, Einc[port[p]]);
  c.k0 = k0;
  c.pad = 0.0;
  *out = c;
}

// ---------------------------------------------------------------------------
// candidate edge lists

__device__ __forceinline__ int flipped_parity(const int *tl, int nf, int t) {
  int p = 0;
  for (int i = 0; i < nf; ++i) p ^= (tl[i] == t);
  return p;
}

// One warp per candidate. Output: es[c*kmax + q], ed[...], ek[c]; ek = -1 on
// an invalid tile index or flip count.
__global__ void k_edge_lists(Geo g, int ncand, Gate gt, const int *__restrict__ tiles, const int *__restrict__ nflip,
                             const int *__restrict__ tile_map, const signed char *__restrict__ P,
                             int *__restrict__ es, signed char *__restrict__ ed, int *__restrict__ ek) {
  extern __shared__ int sh[];
  const int warps = blockDim.x / 32;
  const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int c = blockIdx.x * warps + w;
  const int slots = g.max_flips * ((g.cells_x) * (g.cells_y + 1) + (g.cells_x + 1) * g.cells_y);
  int *cg = sh + w * 2 * slots;          // candidate edge index per slot (-1 = none)
  int *cd = cg + slots;                  // sign per slot
  if (!gt.open(&ncand) || c >= ncand) return;
  const int nfl = nflip[c];
  const int *tl = tiles + (size_t)c * g.max_flips;
  bool bad = nfl < 0 || nfl > g.max_flips;
  for (int i = 0; i < nfl && !bad; ++i) bad = tl[i] < 0 || tl[i] >= g.map_sz;
  if (bad) {
    if (lane == 0) ek[c] = -1;
    return;
  }
  const int nex = g.cells_x * (g.cells_y + 1);
  const int ne = nex + (g.cells_x + 1) * g.cells_y;
  const int total = nfl * ne;
  for (int q = lane; q < total; q += 32) {
    const int t = tl[q / ne], e = q % ne;
    const int ty = t / g.tiles_x, tx = t - ty * g.tiles_x;
    long gi;
    int o1 = t, o2 = -1;
    if (e < nex) {
      const int jj = e / g.cells_x, ii = e % g.cells_x;
      gi = (long)(tx * g.cells_x + ii) + (long)(ty * g.cells_y + jj) * g.ex_xsz;
      if (jj == 0 && ty > 0) o2 = t - g.tiles_x;
      if (jj == g.cells_y && ty + 1 < g.tiles_y) o2 = t + g.tiles_x;
    } else {
      const int e2 = e - nex;
      const int jj = e2 / (g.cells_x + 1), ii = e2 % (g.cells_x + 1);
      gi = g.nx + (long)(tx * g.cells_x + ii) + (long)(ty * g.cells_y + jj) * g.ey_xsz;
      if (ii == 0 && tx > 0) o2 = t - 1;
      if (ii == g.cells_x && tx + 1 < g.tiles_x) o2 = t + 1;
    }
    int pn = tile_map[o1] ^ flipped_parity(tl, nfl, o1);
    if (o2 >= 0) pn |= tile_map[o2] ^ flipped_parity(tl, nfl, o2);
    const int dv = pn - (int)P[gi];
    cg[q] = dv != 0 ? (int)gi : -1;
    cd[q] = dv;
  }
  __syncwarp();
  // Deduplicate (keep first occurrence) and rank by edge index.
  int cnt = 0;
  for (int q = lane; q < total; q += 32) {
    const int gq = cg[q];
    bool keep = gq >= 0;
    for (int r = 0; r < q && keep; ++r) keep = cg[r] != gq;
    if (keep) ++cnt;
  }
  for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  for (int q = lane; q < total; q += 32) {
    const int gq = cg[q];
    bool keep = gq >= 0;
    for (int r = 0; r < q && keep; ++r) keep = cg[r] != gq;
    if (!keep) continue;
    // rank = number of distinct valid edge indices below gq
    int rank = 0;
    for (int r = 0; r < total; ++r) {
      const int gr = cg[r];
      if (gr >= 0 && gr < gq) {
        bool first = true;
        for (int u = 0; u < r && first; ++u) first = cg[u] != gr;
        rank += first;
      }
    }
    if (rank < g.kmax) {
      es[(size_t)c * g.kmax + rank] = gq;
      ed[(size_t)c * g.kmax + rank] = (signed char)cd[q];
    }
  }
  if (lane == 0) ek[c] = cnt <= g.kmax ? cnt : -1;
}

// ---------------------------------------------------------------------------
// cooperative LU of K (column-major, leading dimension ld) in shared memory

// Returns 0 on success, j+1 if pivot j is exactly zero (LAPACK's info).
// Per column j, warp 0 finds the pivot, swaps the rows and scales the column
// (warp shuffles and __syncwarp only), then the whole CTA applies the rank-1
// update of the trailing block: two CTA barriers per column. Every element
// sees the same operations in the same order as in k_eval_warp.
__device__ int cta_lu(double2 *K, int ld, int k, int *piv, double *red_v, int *red_i) {
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ int s_info;
  if (tid == 0) s_info = 0;
  for (int j = 0; j < k; ++j) {
    if (tid < 32) {  // pivot: largest |re|+|im| (first on ties), as izamax
      long long bv = -1;
      int bi = j;
      for (int i = j + tid; i < k; i += 32) {
        const long long v = pivot_key(K[i + j * ld]);
        if (v > bv) { bv = v; bi = i; }
      }
      for (int o = 16; o; o >>= 1) {
        const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
      }
      if (tid == 0) {
        piv[j] = bi;
        red_v[0] = bv >= 0 ? __longlong_as_double(bv) : -1.0;
        if (bv == 0 && s_info == 0) s_info = j + 1;
      }
      if (bi != j)
        for (int c = tid; c < k; c += 32) {
          const double2 t = K[j + c * ld];
          K[j + c * ld] = K[bi + c * ld];
          K[bi + c * ld] = t;
        }
      __syncwarp();
      if (bv != 0) {
        const double2 r = crecip(K[j + j * ld]);
        for (int i = j + 1 + tid; i < k; i += 32) K[i + j * ld] = cmul(K[i + j * ld], r);
      }
    }
    __syncthreads();
    // trailing update: lanes over rows, warps over columns, so that a lane
    // reads its rows' multipliers once per step and the pivot row's entry is
    // a broadcast (the same element operations as any other mapping)
    const int wid = tid >> 5, ln = tid & 31, nw = nt >> 5;
    for (int i = j + 1 + ln; i < k; i += 32) {
      const double2 l = K[i + j * ld];
      for (int c = j + 1 + wid; c < k; c += nw) K[i + c * ld] = cfnma(K[i + c * ld], l, K[j + c * ld]);
    }
    __syncthreads();
  }
  (void)red_i;
  return s_info;
}

// Solves K x = b in place (b in shared memory) with the LU from cta_lu: warp
// 0 alone (the vector is short), then a CTA barrier.
__device__ void cta_lu_solve(const double2 *K, int ld, int k, const int *piv, double2 *b) {
  const int tid = threadIdx.x;
  if (tid < 32) {
    if (tid == 0)
      for (int j = 0; j < k; ++j) {
        const int p = piv[j];
        if (p != j) {
          const double2 t = b[j];
          b[j] = b[p];
          b[p] = t;
        }
      }
    __syncwarp();
    for (int j = 0; j < k; ++j) {  // unit lower
      const double2 bj = b[j];
      for (int i = j + 1 + tid; i < k; i += 32) b[i] = cfnma(b[i], K[i + j * ld], bj);
      __syncwarp();
    }
    for (int j = k - 1; j >= 0; --j) {  // upper
      if (tid == 0) b[j] = cdiv(b[j], K[j + j * ld]);
      __syncwarp();
      const double2 bj = b[j];
      for (int i = tid; i < j; i += 32) b[i] = cfnma(b[i], K[i + j * ld], bj);
      __syncwarp();
    }
  }
  __syncthreads();
}

// Shared prologue of evaluation and accept: gathers K = I + T[s,s] D and
// w = y_s - T[s,s] D Einc_s, factors K, solves K x = w and forms
// z = D (Einc_s + x). Uses shared buffers K (ld x k), vec (k), einc (k),
// piv (k). Returns LAPACK-style info.
template <typename TM>
__device__ int cta_capacitance(const SV<TM> &M, long n, const double2 *__restrict__ Einc,
                               const int *s, const signed char *d, int k, double2 *K, int ld, double2 *vec,
                               double2 *einc, int *piv, double *red) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int c = tid; c < k; c += nt) einc[c] = einc_at(Einc, s[c], n);
  for (int idx = tid; idx < k * k; idx += nt) {
    const int r = idx / k, c = idx % k;  // consecutive threads read along a row of M
    double2 v = M.t(s[r], s[c]);
    if (d[c] < 0) v = make_double2(-v.x, -v.y);
    K[r + c * ld] = v;  // T[s,s] D
  }
  __syncthreads();
  for (int r = tid; r < k; r += nt) {
    double2 w = M.yv(s[r]);
    for (int c = 0; c < k; ++c) w = cfnma(w, K[r + c * ld], einc[c]);
    vec[r] = w;
  }
  __syncthreads();
  for (int r = tid; r < k; r += nt) K[r + r * ld].x += 1.0;
  __syncthreads();
  const int info = cta_lu(K, ld, k, piv, red, nullptr);
  if (info == 0) cta_lu_solve(K, ld, k, piv, vec);
  __syncthreads();
  for (int c = tid; c < k; c += nt) {
    double2 z = cadd(einc[c], vec[c]);
    if (d[c] < 0) z = make_double2(-z.x, -z.y);
    vec[c] = z;
  }
  __syncthreads();
  return info;
}

// ---------------------------------------------------------------------------
// evaluation

// Where the candidate kernels leave each (candidate, frequency)'s factored
// capacitance matrix for the accept: LU (kmax x kmax, column-major, leading
// dimension kmax), row interchanges and z, at slot c * nf + f.
struct LuOut {
  double2 *LU;
  int *piv;
  double2 *z;
};

template <typename TM, int NT>
__global__ void __launch_bounds__(NT) k_eval(const SV<TM> *__restrict__ Ms, const double2 *const *__restrict__ Eincs,
                                              long n, int E, int kmax, const int *__restrict__ es,
                                              const signed char *__restrict__ ed, const int *__restrict__ ek,
                                              const FreqConst *__restrict__ fconst, ObjConst oc, int nf,
                                              double2 *__restrict__ new_eobj, double *__restrict__ Ff,
                                              double *__restrict__ perf, int *__restrict__ status, LuOut lo,
                                              Gate gt) {
  extern __shared__ double2 smem[];
  const int c = blockIdx.x, f = blockIdx.y;
  int ncand = gridDim.x;
  if (!gt.open(&ncand) || c >= ncand) return;
  const int tid = threadIdx.x;
  const int ld = kmax;  // K is kmax x kmax
  double2 *K = smem;
  double2 *vec = K + (size_t)kmax * kmax;
  double2 *einc = vec + kmax;
  int *s = reinterpret_cast<int *>(einc + kmax);
  signed char *d = reinterpret_cast<signed char *>(s + kmax);
  __shared__ int piv[kMaxK];
  __shared__ double red[2];
  __shared__ double2 eo[PNGF_MAX_EOBJ];
  const SV<TM> M = Ms[f];
  const int k = ek[c];
  if (k < 0) {  // invalid candidate
    if (tid == 0) {
      Ff[(size_t)c * nf + f] = nan("");
      status[(size_t)c * nf + f] = PNGF_ERR_ARG;
    }
    return;
  }
  for (int q = tid; q < k; q += blockDim.x) {
    s[q] = es[(size_t)c * kmax + q];
    d[q] = ed[(size_t)c * kmax + q];
  }
  __syncthreads();
  const int info = cta_capacitance(M, n, Eincs[f], s, d, k, K, ld, vec, einc, piv, red);
  if (lo.LU) {  // the factorization, for an accept of this candidate
    const size_t cf = (size_t)c * nf + f;
    double2 *LUo = lo.LU + cf * kmax * kmax;
    for (int idx = tid; idx < k * k; idx += blockDim.x) {
      const int i = idx % k, q = idx / k;
      LUo[i + (size_t)q * kmax] = K[i + q * ld];
    }
    for (int q = tid; q < k; q += blockDim.x) {
      lo.piv[cf * kmax + q] = piv[q];
      lo.z[cf * kmax + q] = vec[q];
    }
  }
  // newEobj = Eobj - R[:,s] z, one warp per objective row.
  const int w = tid / 32, lane = tid % 32;
  for (int e = w; e < E; e += blockDim.x / 32) {
    double2 acc = make_double2(0.0, 0.0);
    for (int q = lane; q < k; q += 32) acc = cadd(acc, cmul(M.r(e, s[q]), vec[q]));
    for (int o = 16; o; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) eo[e] = csub(M.r(e, n), acc);
  }
  __syncthreads();
  if (tid == 0) {
    const size_t cf = (size_t)c * nf + f;
    for (int e = 0; e < E; ++e) new_eobj[cf * E + e] = eo[e];
    double pf[3];
    double F = objective_term(eo, E, fconst[f], oc, pf);
    if (info != 0) F = nan("");
    Ff[cf] = F;
    perf[cf * 3 + 0] = pf[0];
    perf[cf * 3 + 1] = pf[1];
    perf[cf * 3 + 2] = pf[2];
    status[cf] = info != 0 ? PNGF_ERR_SINGULAR : PNGF_OK;
  }
}

// Warp-per-candidate evaluation for candidates of at most 32 edges: WPC warps
// per CTA, one (candidate, frequency) per warp, no CTA-wide barrier. Lane r
// owns row r of K (shared memory, column-major, odd leading dimension) and
// entry r of the edge list, Einc_s and the right-hand side; the pivot search
// is a warp argmax and the triangular solves run in registers with shuffles.
// Every operation, and its order, is the one k_eval performs, so both kernels
// return bit-identical results.
template <typename TM, int WPC>
__global__ void __launch_bounds__(32 * WPC)
    k_eval_warp(const SV<TM> *__restrict__ Ms, const double2 *const *__restrict__ Eincs, long n, int E, int kmax,
                int ncand, const int *__restrict__ es, const signed char *__restrict__ ed,
                const int *__restrict__ ek, const FreqConst *__restrict__ fconst, ObjConst oc, int nf,
                double2 *__restrict__ new_eobj, double *__restrict__ Ff, double *__restrict__ perf,
                int *__restrict__ status, LuOut lo, Gate gt) {
  extern __shared__ double2 smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * WPC + warp, f = blockIdx.y;
  if (!gt.open(&ncand) || c >= ncand) return;
  const int ld = kmax | 1;
  double2 *K = smem + (size_t)warp * ld * kmax;
  const SV<TM> M = Ms[f];
  const int k = ek[c];
  const size_t cf = (size_t)c * nf + f;
  if (k < 0) {
    if (lane == 0) {
      Ff[cf] = nan("");
      status[cf] = PNGF_ERR_ARG;
    }
    return;
  }
  int s_l = 0;
  signed char d_l = 1;
  double2 einc_l = make_double2(0.0, 0.0);
  if (lane < k) {
    s_l = es[(size_t)c * kmax + lane];
    d_l = ed[(size_t)c * kmax + lane];
    einc_l = einc_at(Eincs[f], s_l, n);
  }
  // K = T[s,s] D, one row per step with the lanes along the row.
  for (int r = 0; r < k; ++r) {
    const int sr = __shfl_sync(0xffffffffu, s_l, r);
    if (lane < k) {
      double2 v = M.t(sr, s_l);
      if (d_l < 0) v = make_double2(-v.x, -v.y);
      K[r + lane * ld] = v;
    }
  }
  __syncwarp();
  // w = y_s - T[s,s] D Einc_s, then K += I.
  double2 w = make_double2(0.0, 0.0);
  if (lane < k) w = M.yv(s_l);
  for (int q = 0; q < k; ++q) {
    const double2 eq = shfl2(einc_l, q);
    if (lane < k) w = cfnma(w, K[lane + q * ld], eq);
  }
  if (lane < k) K[lane + lane * ld].x += 1.0;
  __syncwarp();
  // LU with partial pivoting (izamax: largest |re|+|im|, first on ties).
  int info = 0, piv_l = lane;
  for (int j = 0; j < k; ++j) {
    long long bv = -1;
    int bi = j;
    if (lane >= j && lane < k) {
      const long long v = pivot_key(K[lane + j * ld]);
      if (v > bv) {
        bv = v;
        bi = lane;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    const int p = bi;
    if (lane == j) piv_l = p;
    if (bv == 0 && info == 0) info = j + 1;
    if (p != j) {
      if (lane < k) {
        const double2 t = K[j + lane * ld];
        K[j + lane * ld] = K[p + lane * ld];
        K[p + lane * ld] = t;
      }
      __syncwarp();
    }
    if (bv != 0) {
      const double2 r = crecip(K[j + j * ld]);
      if (lane > j && lane < k) K[lane + j * ld] = cmul(K[lane + j * ld], r);
    }
    if (lane > j && lane < k) {
      const double2 l = K[lane + j * ld];
      for (int q = j + 1; q < k; ++q) K[lane + q * ld] = cfnma(K[lane + q * ld], l, K[j + q * ld]);
    }
    __syncwarp();
  }
  if (info == 0) {
    for (int j = 0; j < k; ++j) {  // row interchanges, in order
      const int p = __shfl_sync(0xffffffffu, piv_l, j);
      if (p != j) {
        const double2 bj = shfl2(w, j), bp = shfl2(w, p);
        if (lane == j) w = bp;
        else if (lane == p) w = bj;
      }
    }
    for (int j = 0; j < k; ++j) {  // unit lower
      const double2 bj = shfl2(w, j);
      if (lane > j && lane < k) w = cfnma(w, K[lane + j * ld], bj);
    }
    for (int j = k - 1; j >= 0; --j) {  // upper
      if (lane == j) w = cdiv(w, K[j + j * ld]);
      const double2 bj = shfl2(w, j);
      if (lane < j) w = cfnma(w, K[lane + j * ld], bj);
    }
  }
  double2 z = cadd(einc_l, w);
  if (d_l < 0) z = make_double2(-z.x, -z.y);
  if (lo.LU && lane < k) {  // the factorization, for an accept of this candidate
    const size_t cf = (size_t)c * nf + f;
    double2 *LUo = lo.LU + cf * kmax * kmax;
    for (int q = 0; q < k; ++q) LUo[lane + (size_t)q * kmax] = K[lane + q * ld];
    lo.piv[cf * kmax + lane] = piv_l;
    lo.z[cf * kmax + lane] = z;
  }
  // newEobj = Eobj - R[:,s] z, reduced across the warp as k_eval does.
  double2 eo[PNGF_MAX_EOBJ];
  for (int e = 0; e < E; ++e) {
    double2 acc = make_double2(0.0, 0.0);
    if (lane < k) acc = cadd(acc, cmul(M.r(e, s_l), z));
    for (int o = 16; o; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    eo[e] = csub(M.r(e, n), acc);
  }
  if (lane == 0) {
    for (int e = 0; e < E; ++e) new_eobj[cf * E + e] = eo[e];
    double pf[3];
    double F = objective_term(eo, E, fconst[f], oc, pf);
    if (info != 0) F = nan("");
    Ff[cf] = F;
    perf[cf * 3 + 0] = pf[0];
    perf[cf * 3 + 1] = pf[1];
    perf[cf * 3 + 2] = pf[2];
    status[cf] = info != 0 ? PNGF_ERR_SINGULAR : PNGF_OK;
  }
}

// Sums F over frequencies in frequency order and finds the first candidate
// with F < F_best (a NaN F never passes, as in the reference's compare).
// F_best is read from F_best_dev when that is not null.
__global__ void k_score(int ncand, int nf, const double *__restrict__ Ff, double F_best,
                        const double *__restrict__ F_best_dev, double *__restrict__ F, int *__restrict__ first) {
  __shared__ int s_first;
  if (threadIdx.x == 0) s_first = 0x7fffffff;
  if (F_best_dev) F_best = *F_best_dev;
  __syncthreads();
  for (int c = threadIdx.x; c < ncand; c += blockDim.x) {
    double acc = 0.0;
    for (int f = 0; f < nf; ++f) acc += Ff[(size_t)c * nf + f];
    F[c] = acc;
    if (acc < F_best) atomicMin(&s_first, c);
  }
  __syncthreads();
  if (threadIdx.x == 0) *first = s_first == 0x7fffffff ? -1 : s_first;
}

// Objective of the current state (F of the design M encodes) into F[0],
// per-frequency perf into perf[f*3..].
template <typename TM>
__global__ void k_current_objective(const SV<TM> *__restrict__ Ms, long n, int E,
                                    const FreqConst *__restrict__ fconst, ObjConst oc, int nf, double *F,
                                    double *perf) {
  if (threadIdx.x != 0) return;
  double acc = 0.0;
  for (int f = 0; f < nf; ++f) {
    double2 eo[PNGF_MAX_EOBJ];
    for (int e = 0; e < E; ++e) eo[e] = Ms[f].r(e, n);
    acc += objective_term(eo, E, fconst[f], oc, perf + 3 * f);
  }
  *F = acc;
}

// ---------------------------------------------------------------------------
// accept

// One CTA: factors K for the edge list and stores the LU, pivots and z.
template <typename TM>
__global__ void __launch_bounds__(256) k_acc_factor(const SV<TM> M, long n,
                                                    const double2 *__restrict__ Einc, const int *__restrict__ gs,
                                                    const signed char *__restrict__ gd, int k, double2 *__restrict__ LU,
                                                    int *__restrict__ gpiv, double2 *__restrict__ z,
                                                    int *__restrict__ status, bool check) {
  extern __shared__ double2 smem[];
  double2 *K = smem;
  double2 *vec = K + (size_t)k * k;
  double2 *einc = vec + k;
  int *s = reinterpret_cast<int *>(einc + k);
  signed char *d = reinterpret_cast<signed char *>(s + k);
  __shared__ int piv[kMaxK];
  __shared__ double red[2];
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    s[q] = gs[q];
    d[q] = gd[q];
    // edge lists from a caller (check): every index in [0, n), every sign +-1,
    // before any of them addresses M or Einc
    if (check && (s[q] < 0 || (long)s[q] >= n || (d[q] != 1 && d[q] != -1))) atomicExch(&bad, 1);
  }
  __syncthreads();
  if (bad) {
    if (threadIdx.x == 0) *status = PNGF_ERR_ARG;
    return;
  }
  const int info = cta_capacitance(M, n, Einc, s, d, k, K, k, vec, einc, piv, red);
  for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) LU[idx] = K[idx];
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    gpiv[q] = piv[q];
    z[q] = vec[q];
  }
  if (threadIdx.x == 0 && info != 0) *status = PNGF_ERR_SINGULAR;  // sticky until the host clears it
}

// W[r][j] = d_r (K^-1 M[s, j])_r for j < N, W[r][N] = z_r. One thread per
// column, blockDim.x (32 or 64) columns per CTA; K's LU in shared memory. The
// rows M[s, :] come from Xrows (row r at Xrows + r * ldw, which may be W
// itself: a CTA reads its column block before it writes it) when given, else
// through the view.
template <typename TM>
__global__ void __launch_bounds__(64) k_acc_W(const SV<TM> M, long n, const int *__restrict__ gs,
                                              const signed char *__restrict__ gd, int k, const double2 *__restrict__ LU,
                                              int ldlu, const int *__restrict__ gpiv,
                                              const double2 *__restrict__ z, double2 *W, long ldw,
                                              const int *__restrict__ guard, const double2 *Xrows = nullptr) {
  if (guard && *guard != 0) return;  // the factor step refused the edge list or found K singular
  extern __shared__ double2 smem[];
  double2 *K = smem;                         // k x k
  double2 *X = K + (size_t)k * k;            // k x bw, column j at X[j*k ..]
  const int bw = blockDim.x;
  __shared__ int s[kMaxK];
  __shared__ int piv[kMaxK];
  __shared__ signed char d[kMaxK];
  for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) K[idx] = LU[idx % k + (size_t)(idx / k) * ldlu];
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    s[q] = gs[q];
    piv[q] = gpiv[q];
    d[q] = gd[q];
  }
  __syncthreads();
  const long j0 = (long)blockIdx.x * bw;
  // coalesced load of the column block of rows s
  for (int idx = threadIdx.x; idx < k * bw; idx += blockDim.x) {
    const int r = idx / bw, jj = idx % bw;
    const long j = j0 + jj;
    X[(size_t)jj * k + r] = j >= n ? make_double2(0.0, 0.0) : Xrows ? Xrows[(size_t)r * ldw + j] : M.t(s[r], j);
  }
  __syncthreads();
  const long j = j0 + threadIdx.x;
  double2 *x = X + (size_t)threadIdx.x * k;
  if (j < n) {
    for (int q = 0; q < k; ++q) {
      const int p = piv[q];
      if (p != q) {
        const double2 t = x[q];
        x[q] = x[p];
        x[p] = t;
      }
    }
    for (int q = 0; q < k; ++q) {
      const double2 xq = x[q];
      for (int i = q + 1; i < k; ++i) x[i] = cfnma(x[i], K[i + q * k], xq);
    }
    for (int q = k - 1; q >= 0; --q) {
      const double2 xq = cdiv(x[q], K[q + q * k]);
      x[q] = xq;
      for (int i = 0; i < q; ++i) x[i] = cfnma(x[i], K[i + q * k], xq);
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < k * bw; idx += blockDim.x) {
    const int r = idx / bw, jj = idx % bw;
    const long jw = j0 + jj;
    if (jw < ldw) {
      double2 v;
      if (jw < n) {
        v = X[(size_t)jj * k + r];
        if (d[r] < 0) v = make_double2(-v.x, -v.y);
      } else if (jw == n) {
        v = z[r];
      } else {
        v = make_double2(0.0, 0.0);
      }
      W[(size_t)r * ldw + jw] = v;
    }
  }
}

// Vneg = -D K^-1 (k x k, column-major: Vneg[r + c*k]) from K's LU (LU[i +
// q*ldlu]: unit L below the diagonal, U on and above) and its row interchanges:
// one warp per column c solves K x = e_c (the substitutions of k_acc_W, with
// U's diagonal inverted once). INV_COLS columns per CTA share the LU, staged in
// shared memory so that the sequential steps never wait on global memory.
constexpr int INV_COLS = 2;  // columns of K^-1 per CTA (a warp each): the FP64 solves spread over k / 2 SMs
constexpr int kMaxTcW = 96;  // edges per accept on the tensor-core W path (the LU fits shared memory)
__global__ void __launch_bounds__(32 * INV_COLS) k_acc_inverse(const double2 *__restrict__ LU, int ldlu,
                                                               const int *__restrict__ gpiv,
                                                               const signed char *__restrict__ gd, int k,
                                                               double2 *__restrict__ Vneg) {
  extern __shared__ double2 ism[];
  double2 *K = ism;                            // k x k
  double2 *rdiag = K + (size_t)k * k;          // 1 / U[q][q]
  double2 *xs = rdiag + k;                     // INV_COLS x k
  __shared__ int piv[kMaxK];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int col = w; col < k; col += INV_COLS)  // a warp per column, lanes along it
    for (int r = lane; r < k; r += 32) K[r + (size_t)col * k] = LU[r + (size_t)col * ldlu];
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    piv[q] = gpiv[q];
    rdiag[q] = crecip(LU[q + (size_t)q * ldlu]);
  }
  __syncthreads();
  const int c = blockIdx.x * INV_COLS + w;
  if (c >= k) return;
  double2 *x = xs + (size_t)w * k;
  for (int i = lane; i < k; i += 32) x[i] = make_double2(i == c ? 1.0 : 0.0, 0.0);
  __syncwarp();
  if (lane == 0)
    for (int q = 0; q < k; ++q) {
      const int p = piv[q];
      if (p != q) {
        const double2 t = x[q];
        x[q] = x[p];
        x[p] = t;
      }
    }
  __syncwarp();
  for (int q = 0; q < k; ++q) {
    const double2 xq = x[q];
    for (int i = q + 1 + lane; i < k; i += 32) x[i] = cfnma(x[i], K[i + (size_t)q * k], xq);
    __syncwarp();
  }
  for (int q = k - 1; q >= 0; --q) {
    const double2 xq = cmul(x[q], rdiag[q]);
    __syncwarp();
    if (lane == 0) x[q] = xq;
    for (int i = lane; i < q; i += 32) x[i] = cfnma(x[i], K[i + (size_t)q * k], xq);
    __syncwarp();
  }
  for (int r = lane; r < k; r += 32) {
    const double2 v = x[r];
    Vneg[r + (size_t)c * k] = gd[r] < 0 ? v : make_double2(-v.x, -v.y);
  }
}

// W[r][j] = z_r for j = N, 0 elsewhere (j < ldw): the start of the tensor-core W.
__global__ void k_W_init(double2 *__restrict__ W, long ldw, long n, const double2 *__restrict__ z, int k) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (j < ldw && r < k) W[(size_t)r * ldw + j] = j == n ? z[r] : make_double2(0.0, 0.0);
}

// A[i + r*lda] = M[i][s_r], i < N+E.
template <typename TM>
__global__ void k_acc_gather(const SV<TM> M, long n, long rows, const int *__restrict__ gs, int k,
                             double2 *__restrict__ A, long lda, const int *__restrict__ guard, long row0 = 0) {
  if (guard && *guard != 0) return;
  const long i = row0 + (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  if (i < n)
    for (int r = 0; r < k; ++r) A[(size_t)r * lda + i] = M.t(i, gs[r]);
  else
    for (int r = 0; r < k; ++r) A[(size_t)r * lda + i] = M.r((int)(i - n), gs[r]);
}

// The rows s (ROWS) or the columns s (!ROWS) of T_true = T - U Vt^T for a
// complex64 state with a pending rank-rp correction, as dense FP64 blocks:
//   ROWS:  out[r * ldo + j] = T_true(s_r, j), r < k, j < n;
//   !ROWS: out[c * ldo + i] = T_true(i, s_c), c < k, i < n.
// Reading them through SV::t() costs every element rp loads of a row of Vt
// (or U) 8 * rcap bytes away from its neighbour's; here a CTA stages 64 of
// those rows and the k rows of the other factor in shared memory, 32 ranks at
// a time, and each element's correction is summed in the order and form of
// SV::t(), so the values are bit for bit those read through the view. CTA:
// 64 indices along N (the "many" side), 256 threads, 4 elements each per
// block of 16 edges.
constexpr int PB_M = 64, PB_Q = 32, PB_F = 16;
template <bool ROWS>
__global__ void __launch_bounds__(256) k_pend_block(const float2 *__restrict__ T, long ldt,
                                                    const float2 *__restrict__ U, const float2 *__restrict__ Vt,
                                                    int rcap, int rp, long n, const int *__restrict__ gs, int k,
                                                    double2 *__restrict__ out, long ldo) {
  __shared__ float2 Mc[PB_M][PB_Q + 1];  // padded: lanes read 64-bit words 66 words apart
  __shared__ float2 Fc[PB_F][PB_Q];
  __shared__ int sf[PB_F];
  const long m0 = (long)blockIdx.x * PB_M;
  const int t = threadIdx.x, m = t & (PB_M - 1), fg = t >> 6;  // 4 groups of 4 edges
  const float2 *many = ROWS ? Vt : U, *few = ROWS ? U : Vt;
  for (int fb = 0; fb < k; fb += PB_F) {
    const int nf = min(PB_F, k - fb);
    __syncthreads();
    if (t < PB_F) {
      int e = t < nf ? gs[fb + t] : 0;
      if (!PNGF_BOUNDS_OK(e >= 0 && e < n, kBoundsT, e, 0)) e = 0;
      sf[t] = e;
    }
    float cx[4] = {0.f, 0.f, 0.f, 0.f}, cy[4] = {0.f, 0.f, 0.f, 0.f};
    for (int q0 = 0; q0 < rp; q0 += PB_Q) {
      const int nq = min(PB_Q, rp - q0);
      __syncthreads();  // sf written; the previous chunk consumed
      for (int idx = t; idx < PB_M * PB_Q; idx += 256) {
        const int r = idx / PB_Q, q = idx % PB_Q;
        const long i = m0 + r;
        Mc[r][q] = (i < n && q < nq) ? many[(size_t)i * rcap + q0 + q] : make_float2(0.f, 0.f);
      }
      for (int idx = t; idx < PB_F * PB_Q; idx += 256) {
        const int r = idx / PB_Q, q = idx % PB_Q;
        Fc[r][q] = (r < nf && q < nq) ? few[(size_t)sf[r] * rcap + q0 + q] : make_float2(0.f, 0.f);
      }
      __syncthreads();
      for (int q = 0; q < nq; ++q) {
        const float2 mv = Mc[m][q];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float2 fv = Fc[fg * 4 + u][q];
          // SV::t(): a = U[i][q], b = Vt[j][q]
          const float2 a = ROWS ? fv : mv, b = ROWS ? mv : fv;
          cx[u] = fmaf(a.x, b.x, fmaf(-a.y, b.y, cx[u]));
          cy[u] = fmaf(a.x, b.y, fmaf(a.y, b.x, cy[u]));
        }
      }
    }
    const long i = m0 + m;
    if (i < n) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int f = fg * 4 + u;
        if (f >= nf) continue;
        const float2 tv = ROWS ? T[(size_t)sf[f] * ldt + i] : T[(size_t)i * ldt + sf[f]];
        double2 v = make_double2((double)tv.x, (double)tv.y);
        v.x -= (double)cx[u];
        v.y -= (double)cy[u];
        out[(size_t)(fb + f) * ldo + i] = v;
      }
    }
  }
}

// M[i][j] -= sum_r A[i][r] W[r][j] for i < rows, j < cols. 64x64 tile per
// CTA of 256 threads, 4x4 complex outputs per thread, k in steps of 8.
constexpr int RU_T = 64, RU_KS = 8;
__global__ void __launch_bounds__(256) k_rank_update(double2 *__restrict__ M, long ldm, long rows, long cols,
                                                     const double2 *__restrict__ A, long lda,
                                                     const double2 *__restrict__ W, long ldw, int k,
                                                     const int *__restrict__ guard) {
  if (guard && *guard != 0) return;  // M stays as it was
  __shared__ double2 As[RU_KS][RU_T];
  __shared__ double2 Ws[RU_KS][RU_T];
  const int tid = threadIdx.x;
  const int ti = tid / 16, tj = tid % 16;
  const long i0 = (long)blockIdx.y * RU_T, j0 = (long)blockIdx.x * RU_T;
  double2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0.0, 0.0);
  for (int r0 = 0; r0 < k; r0 += RU_KS) {
    for (int idx = tid; idx < RU_KS * RU_T; idx += 256) {
      const int rr = idx / RU_T, q = idx % RU_T;
      const int r = r0 + rr;
      const long i = i0 + q, j = j0 + q;
      As[rr][q] = (r < k && i < rows) ? A[(size_t)r * lda + i] : make_double2(0.0, 0.0);
      Ws[rr][q] = (r < k && j < cols) ? W[(size_t)r * ldw + j] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int rr = 0; rr < RU_KS; ++rr) {
      double2 a[4], w[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[rr][ti + 16 * q];
        w[q] = Ws[rr][tj + 16 * q];
      }
#pragma unroll
      for (int qa = 0; qa < 4; ++qa)
#pragma unroll
        for (int qb = 0; qb < 4; ++qb) {
          acc[qa][qb].x = fma(a[qa].x, w[qb].x, acc[qa][qb].x);
          acc[qa][qb].x = fma(-a[qa].y, w[qb].y, acc[qa][qb].x);
          acc[qa][qb].y = fma(a[qa].x, w[qb].y, acc[qa][qb].y);
          acc[qa][qb].y = fma(a[qa].y, w[qb].x, acc[qa][qb].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int qa = 0; qa < 4; ++qa) {
    const long i = i0 + ti + 16 * qa;
    if (i >= rows) continue;
#pragma unroll
    for (int qb = 0; qb < 4; ++qb) {
      const long j = j0 + tj + 16 * qb;
      if (j >= cols) continue;
      double2 *p = M + (size_t)i * ldm + j;
      *p = csub(*p, acc[qa][qb]);
    }
  }
}

__global__ void k_commit(int kmax, int c, const int *__restrict__ es, const signed char *__restrict__ ed,
                         const int *__restrict__ ek, int max_flips, const int *__restrict__ tiles,
                         const int *__restrict__ nflip, signed char *__restrict__ P, int *__restrict__ tile_map) {
  const int k = ek[c];
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    const int e = es[(size_t)c * kmax + q];
    P[e] = (signed char)(P[e] + ed[(size_t)c * kmax + q]);
  }
  if (threadIdx.x == 0)
    for (int i = 0; i < nflip[c]; ++i) tile_map[tiles[(size_t)c * max_flips + i]] ^= 1;
}

// ---------------------------------------------------------------------------
// host launchers

static ObjConst obj_const(const Handle *h) { return ObjConst{h->cfg.dx, h->cfg.dy, h->cfg.dz}; }

// Views of frequency f: the FP64 layout (everything in M64) and the complex64
// layout (T in T32, y and R/Eobj in FP64).
// Bounds-checked build: give a view the extents its indices must fall in.
template <typename TM>
static SV<TM> checked(SV<TM> v, long n, int E) {
#ifdef PNGF_BOUNDS_CHECK
  v.bn = n;
  v.be = E;
#else
  (void)n;
  (void)E;
#endif
  return v;
}

static SV<double2> view64(const Handle *h, int f) {
  const double2 *M = h->f[f].M64;
  return checked(SV<double2>{M, h->ldm, M + h->n, h->ldm, M + (size_t)h->n * h->ldm, h->ldm}, h->n, h->E);
}
static SV<float2> view32(const Handle *h, int f) {
  SV<float2> v{h->f[f].T32, h->ldm, h->f[f].y64, 1, h->f[f].R64, h->ldm};
  v.U = h->f[f].U;
  v.Vt = h->f[f].Vt;
  v.rp = h->defer_rp;
  v.rcap = h->defer_cap;
  return checked(v, h->n, h->E);
}

cudaError_t setup_views(Handle *h) {
  const int nf = h->cfg.num_freq;
  if (h->cfg.precision == PNGF_PREC_FP64) {
    std::vector<SV<double2>> v(nf);
    for (int f = 0; f < nf; ++f) v[f] = view64(h, f);
    return cudaMemcpy(h->d_views, v.data(), sizeof(SV<double2>) * nf, cudaMemcpyHostToDevice);
  }
  std::vector<SV<float2>> v(nf);
  for (int f = 0; f < nf; ++f) v[f] = view32(h, f);
  return cudaMemcpy(h->d_views, v.data(), sizeof(SV<float2>) * nf, cudaMemcpyHostToDevice);
}

size_t view_bytes() { return sizeof(SV<double2>) > sizeof(SV<float2>) ? sizeof(SV<double2>) : sizeof(SV<float2>); }

__global__ void k_set_pending_rank(SV<float2> *views, int nf, int rp) {
  if (threadIdx.x < nf) views[threadIdx.x].rp = rp;
}

cudaError_t launch_set_pending_rank(Handle *h) {
  if (h->cfg.precision != PNGF_PREC_C64) return cudaSuccess;
  k_set_pending_rank<<<1, 32, 0, h->stream>>>(static_cast<SV<float2> *>(h->d_views), h->cfg.num_freq, h->defer_rp);
  h->nlaunch += 1;
  return cudaGetLastError();
}

cudaError_t launch_init_M(Handle *h, int f) {
  Freq &q = h->f[f];
  const long n = h->n;
  cudaStream_t st = lane_stream(h, f);
  dim3 tb(32, 8), tg((unsigned)((h->ldm + 31) / 32), (unsigned)((n + 31) / 32));
  k_init_M_tile<<<tg, tb, 0, st>>>(q.G, n, h->ldm, q.M64);
  long *d_port = nullptr;
  cudaError_t e = cudaMallocAsync(&d_port, sizeof(long) * h->port.size(), st);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(d_port, h->port.data(), sizeof(long) * h->port.size(), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  k_init_M_rows<<<(unsigned)((h->ldm + 255) / 256), 256, 0, st>>>(q.G, q.gobj, n, h->E, h->ldm, d_port,
                                                                  (int)h->port.size(), q.M64, q.Einc);
  const double k0 = 2.0 * M_PI * h->cfg.freq_hz[f] / 2.997924579998211e8;
  k_port_const<<<1, 1, 0, st>>>(q.Einc, q.gobj, n, h->E, d_port, (int)h->port.size(), k0, h->d_fconst + f);
  cudaFreeAsync(d_port, st);
  h->nlaunch += 3;
  return cudaGetLastError();
}

cudaError_t launch_edge_lists(Handle *h, int ncand, const int *d_tiles, const int *d_nflip, Gate gt) {
  const Geo g = make_geo(h);
  const int slots = g.max_flips * ((g.cells_x) * (g.cells_y + 1) + (g.cells_x + 1) * g.cells_y);
  const int warps = 4;
  const size_t sm = sizeof(int) * 2 * slots * warps;
  k_edge_lists<<<(ncand + warps - 1) / warps, 32 * warps, sm, h->stream>>>(g, ncand, gt, d_tiles, d_nflip,
                                                                          h->d_tile_map, h->d_P, h->d_es, h->d_ed,
                                                                          h->d_ek);
  h->nlaunch += 1;
  return cudaGetLastError();
}

static size_t eval_smem(int kmax) {
  return sizeof(double2) * ((size_t)kmax * kmax + 2 * kmax) + sizeof(int) * kmax + kmax + 16;
}

template <typename TM, int NT> static cudaError_t launch_eval_cta(Handle *h, int ncand, Gate gt) {
  const int nf = h->cfg.num_freq;
  const size_t sm = eval_smem(h->kmax);
  cudaError_t e = cudaFuncSetAttribute(k_eval<TM, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_eval<TM, NT><<<dim3(ncand, nf), NT, sm, h->stream>>>(
      static_cast<const SV<TM> *>(h->d_views), reinterpret_cast<const double2 *const *>(h->d_Eincs), h->n, h->E,
      h->kmax, h->d_es, h->d_ed, h->d_ek, h->d_fconst, obj_const(h), nf, h->d_new_eobj, h->d_Ff, h->d_perf,
      h->d_status, LuOut{h->d_eval_LU, h->d_eval_piv, h->d_eval_z}, gt);
  return cudaGetLastError();
}

template <typename TM, int WPC> static cudaError_t launch_eval_warp(Handle *h, int ncand, Gate gt) {
  const int nf = h->cfg.num_freq;
  const size_t sm = sizeof(double2) * (size_t)WPC * (h->kmax | 1) * h->kmax;
  cudaError_t e = cudaFuncSetAttribute(k_eval_warp<TM, WPC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_eval_warp<TM, WPC><<<dim3((ncand + WPC - 1) / WPC, nf), 32 * WPC, sm, h->stream>>>(
      static_cast<const SV<TM> *>(h->d_views), reinterpret_cast<const double2 *const *>(h->d_Eincs), h->n, h->E,
      h->kmax, ncand, h->d_es, h->d_ed, h->d_ek, h->d_fconst, obj_const(h), nf, h->d_new_eobj, h->d_Ff, h->d_perf,
      h->d_status, LuOut{h->d_eval_LU, h->d_eval_piv, h->d_eval_z}, gt);
  return cudaGetLastError();
}

bool eval_variant_ok(const Handle *h, int v) {
  if (v < 0 || v >= kEvalVariants) return false;
  return kEvalForms[v].cands_per_cta == 1 || h->kmax <= 32;
}

template <typename TM> static cudaError_t launch_eval_t(Handle *h, int v, int ncand, Gate gt) {
  switch (eval_variant_ok(h, v) ? v : 0) {
    case 1: return launch_eval_cta<TM, 64>(h, ncand, gt);
    case 2: return launch_eval_cta<TM, 256>(h, ncand, gt);
    case 3: return launch_eval_warp<TM, 2>(h, ncand, gt);
    case 4: return launch_eval_warp<TM, 4>(h, ncand, gt);
    case 5: return launch_eval_warp<TM, 8>(h, ncand, gt);
    default: return launch_eval_cta<TM, 128>(h, ncand, gt);
  }
}

cudaError_t launch_eval_form(Handle *h, int form, int ncand, Gate gt) {
  const cudaError_t e = h->cfg.precision == PNGF_PREC_FP64 ? launch_eval_t<double2>(h, form, ncand, gt)
                                                           : launch_eval_t<float2>(h, form, ncand, gt);
  h->nlaunch += 1;
  return e;
}

cudaError_t launch_eval(Handle *h, int ncand, double F_best, const double *d_fbest) {
  const int v = ncand <= kSmallBatch && h->eval_variant_small >= 0 ? h->eval_variant_small : h->eval_variant;
  cudaError_t e = h->cfg.precision == PNGF_PREC_FP64 ? launch_eval_t<double2>(h, v, ncand, Gate{})
                                                     : launch_eval_t<float2>(h, v, ncand, Gate{});
  if (e != cudaSuccess) return e;
  k_score<<<1, 256, 0, h->stream>>>(ncand, h->cfg.num_freq, h->d_Ff, F_best, d_fbest, h->d_F, h->d_first);
  h->nlaunch += 2;
  return cudaGetLastError();
}

cudaError_t launch_current_objective(Handle *h) {
  if (h->cfg.precision == PNGF_PREC_FP64)
    k_current_objective<double2><<<1, 32, 0, h->stream>>>(static_cast<const SV<double2> *>(h->d_views), h->n, h->E,
                                                          h->d_fconst, obj_const(h), h->cfg.num_freq, h->d_F,
                                                          h->d_perf);
  else
    k_current_objective<float2><<<1, 32, 0, h->stream>>>(static_cast<const SV<float2> *>(h->d_views), h->n, h->E,
                                                         h->d_fconst, obj_const(h), h->cfg.num_freq, h->d_F,
                                                         h->d_perf);
  h->nlaunch += 1;
  return cudaGetLastError();
}

// Accept prologue on either layout: K's LU and z, W = [D K^-1 T[s,:], z],
// A = [T; R][:, s] (FP64, column-major with leading dimension N+E).
template <typename TM>
static cudaError_t accept_prologue(const SV<TM> &v, long n, int E, long ldm, const double2 *Einc, const int *d_s,
                                   const signed char *d_d, int k, double2 *LU, int *piv, double2 *z, double2 *A,
                                   double2 *W, int *status, cudaStream_t stream, const LuOut *given = nullptr,
                                   int ld_given = 0, bool raw = false) {
  const long rows = n + E;
  const double2 *lu = LU, *zz = z;
  const int *pv = piv;
  int ldlu = k;
  cudaError_t e;
  if (given) {  // the factorization the candidate kernel left (leading dimension ld_given)
    lu = given->LU;
    pv = given->piv;
    zz = given->z;
    ldlu = ld_given;
  } else {
    const size_t smf = sizeof(double2) * ((size_t)k * k + 2 * k) + sizeof(int) * k + k + 16;
    e = cudaFuncSetAttribute(k_acc_factor<TM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smf);
    if (e != cudaSuccess) return e;
    k_acc_factor<TM><<<1, 256, smf, stream>>>(v, n, Einc, d_s, d_d, k, LU, piv, z, status, raw);
  }
  const int wc = k <= 64 ? 64 : 32;  // columns per CTA, so that K and the block fit in shared memory
  const size_t smw = sizeof(double2) * ((size_t)k * k + (size_t)k * wc);
  e = cudaFuncSetAttribute(k_acc_W<TM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smw);
  if (e != cudaSuccess) return e;
  // raw (caller-owned buffers): the later kernels skip their work once the
  // factor step has set the status, so that M is left as it was
  const int *guard = raw ? status : nullptr;
  if constexpr (std::is_same<TM, float2>::value) {
    if (v.rp > 0 && !raw) {
      // a pending correction: the rows s of T_true into W (read back by
      // k_acc_W) and its columns s into A, each element's correction summed
      // once; then the objective rows of A from the view
      const unsigned gb = (unsigned)((n + PB_M - 1) / PB_M);
      k_pend_block<true><<<gb, 256, 0, stream>>>(v.T, v.ldt, v.U, v.Vt, v.rcap, v.rp, n, d_s, k, W, ldm);
      k_acc_W<TM><<<(unsigned)((ldm + wc - 1) / wc), wc, smw, stream>>>(v, n, d_s, d_d, k, lu, ldlu, pv, zz, W,
                                                                        ldm, guard, W);
      k_pend_block<false><<<gb, 256, 0, stream>>>(v.T, v.ldt, v.U, v.Vt, v.rcap, v.rp, n, d_s, k, A, rows);
      if (rows > n)
        k_acc_gather<TM><<<(unsigned)((rows - n + 255) / 256), 256, 0, stream>>>(v, n, rows, d_s, k, A, rows, guard,
                                                                                 n);
      return cudaGetLastError();
    }
  }
  k_acc_W<TM><<<(unsigned)((ldm + wc - 1) / wc), wc, smw, stream>>>(v, n, d_s, d_d, k, lu, ldlu, pv, zz, W, ldm,
                                                                    guard);
  k_acc_gather<TM><<<(unsigned)((rows + 255) / 256), 256, 0, stream>>>(v, n, rows, d_s, k, A, rows, guard);
  return cudaGetLastError();
}

// The common start of the tensor-core accept prologues: K's LU and z (those
// the candidate kernel left, for a candidate of the evaluated batch, else
// factored here through the view), Vneg = -D K^-1 into the lane's V, and W
// set to [0, z] (its T part is then accumulated by tensor-core products).
template <typename TM>
static cudaError_t accept_tc_start(Handle *h, int f, const SV<TM> &v, const double2 *Einc, const int *d_s,
                                   const signed char *d_d, int k) {
  const long n = h->n;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  cudaError_t e;
  const double2 *LU = L.LU, *z = L.z;
  const int *piv = L.piv;
  int ldlu = k;
  if (h->acc_cand >= 0) {  // a candidate of the evaluated batch: its kernel left K's LU and z
    const size_t cf = (size_t)h->acc_cand * h->cfg.num_freq + f, km = (size_t)h->kmax;
    LU = h->d_eval_LU + cf * km * km;
    piv = h->d_eval_piv + cf * km;
    z = h->d_eval_z + cf * km;
    ldlu = h->kmax;
  } else {
    const size_t smf = sizeof(double2) * ((size_t)k * k + 2 * k) + sizeof(int) * k + k + 16;
    if ((e = cudaFuncSetAttribute(k_acc_factor<TM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smf)) !=
        cudaSuccess)
      return e;
    k_acc_factor<TM><<<1, 256, smf, st>>>(v, n, Einc, d_s, d_d, k, L.LU, L.piv, L.z, h->d_acc_status, false);
    h->nlaunch += 1;
  }
  const size_t smi = sizeof(double2) * ((size_t)k * k + k + (size_t)INV_COLS * k);
  if ((e = cudaFuncSetAttribute(k_acc_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smi)) != cudaSuccess)
    return e;
  k_acc_inverse<<<(unsigned)((k + INV_COLS - 1) / INV_COLS), 32 * INV_COLS, smi, st>>>(LU, ldlu, piv, d_d, k, L.V);
  k_W_init<<<dim3((unsigned)((h->ldm + 255) / 256), (unsigned)k), 256, 0, st>>>(L.W, h->ldm, n, z, k);
  h->nlaunch += 2;
  return cudaGetLastError();
}

// Accept prologue with W on the tensor cores: K's LU and z (those the candidate
// kernel left, for a candidate of the evaluated batch), Vneg = -D K^-1,
// W = [D K^-1 T[s, 0:N], z] as Vneg times the rows s of the state with the
// FP64-accurate tensor-core product, A = [T; R][:, s]. For the FP64 layout and
// the complex64 one without deferred updates (whose rows are read as stored).
template <typename TM>
static cudaError_t accept_prologue_tc(Handle *h, int f, const SV<TM> &v, const void *X, bool x32,
                                      const double2 *Einc, const int *d_s, const signed char *d_d, int k) {
  const long n = h->n, rows = n + h->E;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  cudaError_t e;
  if ((e = accept_tc_start<TM>(h, f, v, Einc, d_s, d_d, k)) != cudaSuccess) return e;
  if ((e = launch_f64tc_wgemm(h, f, k, L.V, X, x32, h->ldm, d_s, L.W)) != cudaSuccess) return e;
  k_acc_gather<TM><<<(unsigned)((rows + 255) / 256), 256, 0, st>>>(v, n, rows, d_s, k, L.A, rows, nullptr);
  h->nlaunch += 1;
  return cudaGetLastError();
}

// FP64 accepts of more than f64tc_max_k() edges: the rows s of the state as
// a dense block, Xs[r][j] = T[s_r][j] (j < N), and K D = T[s,s] + D
// (column-major k x k), for the refinement of W below.
__global__ void k_rows_kd(const SV<double2> M, long n, const int *__restrict__ gs,
                          const signed char *__restrict__ gd, int k, double2 *__restrict__ Xs, long ldx,
                          double2 *__restrict__ KD) {
  const int r = blockIdx.y;
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= k || j >= n) return;
  const int sr = gs[r];
  Xs[(size_t)r * ldx + j] = M.t(sr, j);
  if (j < k) {  // column c = j of K D
    double2 v = M.t(sr, gs[j]);
    if (j == r) v.x += (double)gd[j];
    KD[r + (size_t)j * k] = v;
  }
}

// Accept prologue of an FP64 accept of more than f64tc_max_k() (and at most
// kMaxTcW) edges with W on the tensor cores: W0 = -Vneg X with the explicit
// inverse, then one step of refinement, W = W0 - Vneg (X - K D W0), all three
// products FP64-accurate on the tensor cores. An explicit inverse alone is
// not backward stable (at 96 edges it cost a factor of about 10 in the
// state's error); the refinement step brings W back to the accuracy of
// triangular solves, which on GB300's narrow FP64 pipe (one thread per
// column of W) took longer than the three products together.
static cudaError_t accept_prologue_tc_refined(Handle *h, int f, const SV<double2> &v, const double2 *Einc,
                                              const int *d_s, const signed char *d_d, int k) {
  const long n = h->n, rows = n + h->E;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  cudaError_t e;
  if ((e = accept_tc_start<double2>(h, f, v, Einc, d_s, d_d, k)) != cudaSuccess) return e;
  k_rows_kd<<<dim3((unsigned)((n + 255) / 256), (unsigned)k), 256, 0, st>>>(v, n, d_s, d_d, k, L.Xs, h->ldm, L.KD);
  h->nlaunch += 1;
  if ((e = launch_f64tc_wgemm(h, f, k, L.V, v.T, false, h->ldm, d_s, L.W)) != cudaSuccess) return e;  // W0
  if ((e = launch_f64tc_small(h, f, k, L.Xs, k, n, h->ldm, L.KD, k, L.W, h->ldm)) != cudaSuccess)
    return e;  // Xs = X - K D W0
  if ((e = launch_f64tc_small(h, f, k, L.W, k, n, h->ldm, L.V, k, L.Xs, h->ldm)) != cudaSuccess)
    return e;  // W = W0 - Vneg (X - K D W0)
  k_acc_gather<double2><<<(unsigned)((rows + 255) / 256), 256, 0, st>>>(v, n, rows, d_s, k, L.A, rows, nullptr);
  h->nlaunch += 1;
  return cudaGetLastError();
}

// The same with a pending correction (deferred complex64): the rows s of
// T_true are formed densely first (k_pend_block, in the lane's Xs) and the
// tensor-core product reads them in place of the stored rows; A's T part is
// the dense block of columns s, its objective rows come through the view.
static cudaError_t accept_prologue_tc_pend(Handle *h, int f, const SV<float2> &v, const double2 *Einc,
                                           const int *d_s, const signed char *d_d, int k) {
  const long n = h->n, rows = n + h->E;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  cudaError_t e;
  if ((e = accept_tc_start<float2>(h, f, v, Einc, d_s, d_d, k)) != cudaSuccess) return e;
  const unsigned gb = (unsigned)((n + PB_M - 1) / PB_M);
  k_pend_block<true><<<gb, 256, 0, st>>>(v.T, v.ldt, v.U, v.Vt, v.rcap, v.rp, n, d_s, k, L.Xs, h->ldm);
  h->nlaunch += 1;
  if ((e = launch_f64tc_wgemm(h, f, k, L.V, L.Xs, false, h->ldm, h->d_iota, L.W)) != cudaSuccess) return e;
  k_pend_block<false><<<gb, 256, 0, st>>>(v.T, v.ldt, v.U, v.Vt, v.rcap, v.rp, n, d_s, k, L.A, rows);
  if (rows > n)
    k_acc_gather<float2><<<(unsigned)((rows - n + 255) / 256), 256, 0, st>>>(v, n, rows, d_s, k, L.A, rows, nullptr,
                                                                            n);
  h->nlaunch += 2;
  return cudaGetLastError();
}

cudaError_t launch_accept_edges(Handle *h, int f, const int *d_s, const signed char *d_d, int k, int layout) {
  Freq &q = h->f[f];
  const long n = h->n, rows = n + h->E;
  if (k <= 0) return cudaSuccess;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  cudaError_t e;
  // complex64 with nothing pending (no deferral, a build, or the first accept
  // after a flush): W on the tensor cores from the rows of T32 as stored;
  // with pending deferred updates from the dense rows of T_true (the FP64
  // triangular solves below remain for larger edge lists)
  if (h->f64tc && layout == PNGF_PREC_C64 && (h->defer_cap == 0 || h->defer_rp == 0) && k <= kMaxTcW) {
    if ((e = accept_prologue_tc<float2>(h, f, view32(h, f), q.T32, true, q.Einc, d_s, d_d, k)) != cudaSuccess)
      return e;
    return h->defer_now ? launch_c64_defer(h, f, k) : launch_c64_update(h, f, k);
  }
  // with pending deferred updates: the same, from dense rows of T_true
  if (h->f64tc && layout == PNGF_PREC_C64 && L.Xs && h->d_iota && k <= kMaxTcW && k <= h->acc_cap) {
    if ((e = accept_prologue_tc_pend(h, f, view32(h, f), q.Einc, d_s, d_d, k)) != cudaSuccess) return e;
    return h->defer_now ? launch_c64_defer(h, f, k) : launch_c64_update(h, f, k);
  }
  // FP64: W from K's explicit inverse only up to f64tc_max_k() edges; above,
  // its error grows with cond(K) beyond that of the triangular solves
  // (which the larger accepts keep), while the update itself runs on the
  // tensor cores in pieces either way
  if (h->f64tc && layout != PNGF_PREC_C64 && k <= f64tc_max_k()) {
    if ((e = accept_prologue_tc<double2>(h, f, view64(h, f), q.M64, false, q.Einc, d_s, d_d, k)) != cudaSuccess)
      return e;
    return launch_f64tc_update(h, f, k, q.M64, L.A, L.W);
  }
  // larger FP64 accepts: the explicit inverse and one refinement step
  if (h->f64tc && layout != PNGF_PREC_C64 && L.Xs && L.KD && k <= kMaxTcW && k <= h->acc_cap) {
    if ((e = accept_prologue_tc_refined(h, f, view64(h, f), q.Einc, d_s, d_d, k)) != cudaSuccess) return e;
    return launch_f64tc_update(h, f, k, q.M64, L.A, L.W);
  }
  // a candidate of the evaluated batch: start from the factorization its kernel left
  LuOut ev{};
  const LuOut *given = nullptr;
  if (h->acc_cand >= 0) {
    const size_t cf = (size_t)h->acc_cand * h->cfg.num_freq + f, km = (size_t)h->kmax;
    ev = LuOut{h->d_eval_LU + cf * km * km, h->d_eval_piv + cf * km, h->d_eval_z + cf * km};
    given = &ev;
  }
  if (layout == PNGF_PREC_C64) {
    e = accept_prologue<float2>(view32(h, f), n, h->E, h->ldm, q.Einc, d_s, d_d, k, L.LU, L.piv, L.z, L.A, L.W,
                                h->d_acc_status, st, given, h->kmax);
    if (e != cudaSuccess) return e;
    h->nlaunch += 3;
    return h->defer_now ? launch_c64_defer(h, f, k) : launch_c64_update(h, f, k);
  }
  e = accept_prologue<double2>(view64(h, f), n, h->E, h->ldm, q.Einc, d_s, d_d, k, L.LU, L.piv, L.z, L.A, L.W,
                               h->d_acc_status, st, given, h->kmax);
  if (e != cudaSuccess) return e;
  if (h->f64tc) {  // W by FP64 solves, the update on the tensor cores
    h->nlaunch += 3;
    return launch_f64tc_update(h, f, k, q.M64, L.A, L.W);
  }
  dim3 g((unsigned)((n + 1 + RU_T - 1) / RU_T), (unsigned)((rows + RU_T - 1) / RU_T));
  cudaEvent_t t0 = timing_mark(h, st);
  k_rank_update<<<g, 256, 0, st>>>(q.M64, h->ldm, rows, n + 1, L.A, rows, L.W, h->ldm, k, nullptr);
  const double cells = (double)rows * (double)(n + 1);
  timing_close(h, t0, T_UPDATE, 8.0 * k * cells, 2.0 * 16.0 * cells + 16.0 * k * (double)(rows + n + 1), 0.0, st);
  h->nlaunch += 4;
  return cudaGetLastError();
}

cudaError_t launch_accept_raw(double2 *M, long ldm, long n, int E, const double2 *Einc, const int *d_s,
                              const signed char *d_d, int k, double2 *LU, int *piv, double2 *z, double2 *A,
                              double2 *W, int *status, cudaStream_t stream) {
  const long rows = n + E;
  if (k <= 0) return cudaSuccess;
  const SV<double2> v = checked(SV<double2>{M, ldm, M + n, ldm, M + (size_t)n * ldm, ldm}, n, E);
  cudaError_t e =
      accept_prologue<double2>(v, n, E, ldm, Einc, d_s, d_d, k, LU, piv, z, A, W, status, stream, nullptr, 0, true);
  if (e != cudaSuccess) return e;
  dim3 g((unsigned)((n + 1 + RU_T - 1) / RU_T), (unsigned)((rows + RU_T - 1) / RU_T));
  k_rank_update<<<g, 256, 0, stream>>>(M, ldm, rows, n + 1, A, rows, W, ldm, k, status);
  return cudaGetLastError();
}

cudaError_t bounds_read_fp64(long long out[4], bool reset) {
#ifdef PNGF_BOUNDS_CHECK
  return bounds_read_tu(out, reset);
#else
  (void)reset;
  for (int q = 0; q < 4; ++q) out[q] = 0;
  return cudaSuccess;
#endif
}

cudaError_t launch_commit(Handle *h, int c) {
  k_commit<<<1, 128, 0, h->stream>>>(h->kmax, c, h->d_es, h->d_ed, h->d_ek, h->cfg.max_flips, h->d_tiles,
                                      h->d_nflip, h->d_P, h->d_tile_map);
  h->nlaunch += 1;
  return cudaGetLastError();
}

}  // namespace pngf
