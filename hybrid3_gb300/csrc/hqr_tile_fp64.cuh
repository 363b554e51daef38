// hqr_tile_fp64.cuh -- FP64 tile kernels of the tiled Householder QR, run by
// one CTA of kThreads threads on CUDA cores.
//
// These restate, as block-cooperative CUDA, the four PLASMA CORE kernels that
// Hybrid_tile_QR calls (Hybrid_tile_QR.c:985 CORE_dgeqrt, :1135 CORE_dtsqrt,
// :1276 CORE_dormqr, :1356 CORE_dtsmqr):
//   * reflectors follow LAPACK dlarfg: beta = -sign(alpha)*||[alpha; x]||,
//     tau = 0 when x = 0, with the safe-minimum rescaling for tiny columns;
//   * the factorization and its updates run in w-column inner blocks
//     (w = min(IB, 32)); each block's w x w upper-triangular T is stored as a
//     diagonal block of the panel tile's NB x NB T (the full T, whose diagonal
//     w x w blocks are exactly the IB-blocked T of the LAPACK dgeqrt layout);
//   * a block reflector is applied as W = V^T C, W = T^T W, C -= V W.
//
// Shared memory holds the panel / the column block being updated; V and T are
// streamed from global memory (L2) in row chunks.  FP64 throughput on GB300 is
// ~1 TFLOP/s per GPU, so the kernels are FP64-issue bound and favour simple
// conflict-free shared-memory access over register blocking.
#pragma once
#include <cfloat>
#include "hqr_common.cuh"

namespace hqr {

constexpr int kMaxW = 32;      // inner block width
constexpr int kRC = 128;       // V row chunk staged per pass
constexpr int kRedSlots = 32;  // block-reduction scratch: kWarps partials, then 4 broadcasts
constexpr int kBcast = kWarps; // first broadcast slot
constexpr int kSplitItems = 256;   // at most this many (output, split) items in W = V^T C
static_assert(kWarps + 4 <= kRedSlots, "reduction scratch");

// Shape of the tile kernels for one (NB, IB) configuration.
struct TileShape {
  int NB;   // tile order
  int w;    // inner block width = min(IB, kMaxW)
  int CB;   // columns per LARFB/SSRFB column-block task
  int RC;   // V row chunk
};

// Shared-memory carve-up, in doubles.  Computed identically on host and device.
struct SmemPlan {
  int off_c1, off_c2, off_vb, off_vt, off_t, off_g, off_w, off_w2, off_part, off_red, off_tau;
  int total;
  __host__ __device__ static SmemPlan make(const TileShape& s) {
    SmemPlan p;
    const int NB = s.NB, w = s.w, CB = s.CB;
    // One region serves, one at a time: the GEQRT/TSQRT panel (NB x w), the
    // LARFB column block (NB x CB), the SSRFB pair A1|A2 (2 x NB x CB) and the
    // TSQRT trailing chunk R-rows|A2 (w x CB + NB x CB).
    int region = NB * w;
    if (2 * NB * CB > region) region = 2 * NB * CB;
    if (w * CB + NB * CB > region) region = w * CB + NB * CB;
    int o = 0;
    p.off_c1 = o;
    p.off_c2 = o + NB * CB;                // SSRFB A2
    o += region;
    p.off_vb = o; o += (s.RC + 1) * w;     // V row chunk (ld RC+1)
    p.off_vt = o; o += w * w;              // unit-lower top of V / TSQRT R block
    p.off_t = o; o += w * w;               // T block
    p.off_g = o; o += w * w;               // Gram scratch of the T-block build
    p.off_w = o; o += w * CB;
    p.off_w2 = o; o += w * CB;
    p.off_part = o; o += 8 * kSplitItems;  // split-K partials (<= kSplitItems items x 8)
    p.off_red = o; o += kRedSlots;         // block reductions (kWarps) + broadcasts (4)
    p.off_tau = o; o += kMaxW;
    p.total = o;
    return p;
  }
};

// ---------------------------------------------------------------------------
// Reflector generation (LAPACK dlarfg), block-cooperative.
// alpha: shared scalar; x: shared vector of n elements (unit stride).
// On return *alpha = beta, x is scaled to v(1:n), *tau_out = tau.
// ---------------------------------------------------------------------------
// Range constants of the panel arithmetic R (double; float for the FP32-class
// panels of HQR_PREC_FP32): the smallest normal number and the unit roundoff
// of dlarfg's safe minimum, the magnitudes whose squares stay in range (plain
// path), and the range of a sum of squares whose square root needs no
// scaling.  The panel kernels hold their tile in shared memory as R and
// convert once on the way in and out (the stored values are R's).
template <typename R> struct PanelReal;
template <> struct PanelReal<double> {
  static constexpr double kMin = DBL_MIN, kEps = DBL_EPSILON, kBig = 1e140, kTiny = 1e-140;
  static constexpr double kSsLo = 1e-290, kSsHi = 1e290;
};
template <> struct PanelReal<float> {
  static constexpr float kMin = FLT_MIN, kEps = FLT_EPSILON, kBig = 1e17f, kTiny = 1e-17f;
  static constexpr float kSsLo = 1e-34f, kSsHi = 1e34f;
};

template <typename R>
__device__ __forceinline__ R block_max(R v, R* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  R s = R(0);
#pragma unroll
  for (int i = 0; i < kWarps; i++) s = fmax(s, red[i]);
  return s;
}

// The scalar part of dlarfg for alpha = a, ||x|| = xnorm, ss = ||x||^2; plain:
// ss lies where its square root needs no scaling.  beta = -sign(a) ||[a; x]||,
// tau = (beta - a) / beta, scal = 1 / (a - beta) (x is scaled by scal after
// knt rescalings by 1/safmin, as LAPACK does for tiny columns).
template <typename R>
__device__ __forceinline__ void larfg_scalars(R a, R xnorm, R ss, bool plain, R& tau, R& scal, int& knt,
                                              R& beta) {
  using K = PanelReal<R>;
  tau = R(0);
  beta = a;
  scal = R(1);
  knt = 0;
  const R aa = fabs(a);
  if (xnorm != R(0) && plain && aa < K::kBig && (aa > K::kTiny || a == R(0))) {
    // dlapy2(alpha, ||x||) as sqrt(alpha^2 + ||x||^2): no overflow or
    // underflow in this range, one square root instead of two
    beta = -copysign(sqrt(fma(a, a, ss)), a);
    tau = (beta - a) / beta;
    scal = R(1) / (a - beta);
  } else if (xnorm != R(0)) {
    const R safmin = K::kMin / (K::kEps * R(0.5));
    const R rsafmn = R(1) / safmin;
    R xn = xnorm;
    beta = -copysign(hypot(a, xn), a);
    while (fabs(beta) < safmin && knt < 20) {
      knt++;
      a *= rsafmn;
      xn *= rsafmn;
      beta = -copysign(hypot(a, xn), a);
    }
    tau = (beta - a) / beta;
    scal = R(1) / (a - beta);
    for (int j = 0; j < knt; j++) beta *= safmin;
  }
}

__device__ void block_larfg(double* alpha, double* x, int n, double* tau_out, double* red) {
  double ss = 0.0;
  for (int r = threadIdx.x; r < n; r += kThreads) {
    const double v = x[r];
    ss = fma(v, v, ss);
  }
  ss = block_sum(ss, red);
  double xnorm;
  bool plain = false;   // ||x||^2 and alpha^2 in range: beta from the squared norms directly
  if (ss == 0.0) {
    xnorm = 0.0;
  } else if (ss >= 1e-290 && ss <= 1e290) {
    xnorm = sqrt(ss);
    plain = true;
  } else {  // scaled norm, as LAPACK dnrm2 does, for tiny or huge columns
    double amax = 0.0;
    for (int r = threadIdx.x; r < n; r += kThreads) amax = fmax(amax, fabs(x[r]));
    amax = block_max(amax, red);
    double s2 = 0.0;
    for (int r = threadIdx.x; r < n; r += kThreads) {
      const double v = x[r] / amax;
      s2 = fma(v, v, s2);
    }
    s2 = block_sum(s2, red);
    xnorm = amax * sqrt(s2);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tau, scal, beta;
    int knt;
    larfg_scalars(*alpha, xnorm, ss, plain, tau, scal, knt, beta);
    red[kBcast + 0] = tau;
    red[kBcast + 1] = scal;
    red[kBcast + 2] = (double)knt;
    red[kBcast + 3] = beta;
  }
  __syncthreads();
  const double tau = red[kBcast + 0], scal = red[kBcast + 1];
  const int knt = (int)red[kBcast + 2];
  if (tau != 0.0) {
    const double rsafmn = 1.0 / (DBL_MIN / (DBL_EPSILON * 0.5));
    for (int r = threadIdx.x; r < n; r += kThreads) {
      double v = x[r];
      for (int j = 0; j < knt; j++) v *= rsafmn;
      x[r] = v * scal;
    }
  }
  if (threadIdx.x == 0) {
    *alpha = red[kBcast + 3];
    *tau_out = tau;
  }
  __syncthreads();
}

// dlarfg on [alpha; x] by one warp (x: n contiguous shared doubles), with the
// arithmetic of block_larfg; every lane computes the (identical) scalars.
template <typename R>
__device__ void warp_larfg(R* alpha, R* x, int n, R* tau_out) {
  using K = PanelReal<R>;
  const int lane = threadIdx.x & 31;
  R ss = R(0);
  for (int r = lane; r < n; r += 32) {
    const R v = x[r];
    ss = fma(v, v, ss);
  }
  ss = warp_sum(ss);
  R xnorm;
  bool plain = false;
  if (ss == R(0)) {
    xnorm = R(0);
  } else if (ss >= K::kSsLo && ss <= K::kSsHi) {
    xnorm = sqrt(ss);
    plain = true;
  } else {
    R amax = R(0);
    for (int r = lane; r < n; r += 32) amax = fmax(amax, fabs(x[r]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    R s2 = R(0);
    for (int r = lane; r < n; r += 32) {
      const R v = x[r] / amax;
      s2 = fma(v, v, s2);
    }
    s2 = warp_sum(s2);
    xnorm = amax * sqrt(s2);
  }
  R tau, scal, beta;
  int knt;
  larfg_scalars(*alpha, xnorm, ss, plain, tau, scal, knt, beta);
  if (tau != R(0)) {
    const R rsafmn = R(1) / (K::kMin / (K::kEps * R(0.5)));
    for (int r = lane; r < n; r += 32) {
      R v = x[r];
      for (int j = 0; j < knt; j++) v *= rsafmn;
      x[r] = v * scal;
    }
  }
  __syncwarp();
  if (lane == 0) {
    *alpha = beta;
    *tau_out = tau;
  }
  __syncwarp();
}

// The warp that runs work item `it` of a panel column step: item 0 (the next
// column, whose reflector is on the critical path) has warp 0 to itself, the
// other items go round the remaining warps.
__device__ __forceinline__ bool panel_item_mine(int it, int warp) {
  return it == 0 ? warp == 0 : (warp != 0 && (it - 1) % (kWarps - 1) == warp - 1);
}

// Unblocked QR of the triangle-on-square panel [R; A] (R w x w, upper part
// used; A m x w dense), the per-column loop of CORE_dtsqrt, with the Gram
// matrix of the reflectors for the T build: G(b, c) = v_b . v_c, b < c (ld w).
// Column c's reflector acts on [R(c,c); A(:,c)]; A(:, c) becomes v_c.  At
// step c, the warp that applies reflector c to column c + 1 also forms
// reflector c + 1 (warp_larfg), the other warps apply reflector c to the
// remaining columns and compute G(:, c): one barrier per column.
template <typename RT = double>
__device__ void panel_qr_ts_fused(RT* R, int ldr, RT* A, int lda, int m, int w, RT* tau,
                                  RT* G) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) warp_larfg(R, A, m, tau);
  __syncthreads();
  for (int c = 0; c < w; c++) {
    const RT t = tau[c];
    const RT* ac = A + (size_t)c * lda;
    const int nupd = w - 1 - c;   // items 0..nupd-1: columns c+1..w-1; then G(b, c), b < c
    for (int it = 0; it < nupd + c; it++) {
      if (!panel_item_mine(it, warp)) continue;
      if (it < nupd) {
        const int j = c + 1 + it;
        RT* aj = A + (size_t)j * lda;
        if (t != RT(0)) {
          RT* rcj = R + c + (size_t)j * ldr;
          const RT r0 = *rcj;
          RT s = RT(0);
          for (int r = lane; r < m; r += 32) s = fma(ac[r], aj[r], s);
          s = (warp_sum(s) + r0) * t;
          if (lane == 0) *rcj = r0 - s;
          for (int r = lane; r < m; r += 32) aj[r] = fma(-s, ac[r], aj[r]);
        }
        if (it == 0) {
          __syncwarp();
          warp_larfg(R + j + (size_t)j * ldr, aj, m, tau + j);
        }
      } else {
        const int b = it - nupd;
        const RT* vb = A + (size_t)b * lda;
        RT s = RT(0);
        for (int r = lane; r < m; r += 32) s = fma(vb[r], ac[r], s);
        s = warp_sum(s);
        if (lane == 0) G[b + c * w] = s;
      }
    }
    __syncthreads();
  }
}

// Unblocked QR of a shared panel (dgeqr2 semantics, P m x w, ld ldp, m >= w)
// with the Gram matrix of the unit-lower reflectors, G(b, c) = v_b . v_c =
// P(c, b) + sum_{r > c} P(r, b) P(r, c), b < c (ld w); the same one-barrier
// column step as panel_qr_ts_fused.
template <typename RT = double>
__device__ void panel_qr_ge_fused(RT* P, int ldp, int m, int w, RT* tau, RT* G) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) warp_larfg(P, P + 1, m - 1, tau);
  __syncthreads();
  for (int c = 0; c < w; c++) {
    const RT t = tau[c];
    const RT* pc = P + (size_t)c * ldp;
    const int nupd = w - 1 - c;
    for (int it = 0; it < nupd + c; it++) {
      if (!panel_item_mine(it, warp)) continue;
      if (it < nupd) {
        const int j = c + 1 + it;
        RT* pj = P + (size_t)j * ldp;
        if (t != RT(0)) {
          const RT pcj = pj[c];
          RT s = RT(0);
          for (int r = c + 1 + lane; r < m; r += 32) s = fma(pc[r], pj[r], s);
          s = (warp_sum(s) + pcj) * t;
          if (lane == 0) pj[c] = pcj - s;
          for (int r = c + 1 + lane; r < m; r += 32) pj[r] = fma(-s, pc[r], pj[r]);
        }
        if (it == 0) {
          __syncwarp();
          warp_larfg(pj + j, pj + j + 1, m - j - 1, tau + j);
        }
      } else {
        const int b = it - nupd;
        const RT* pb = P + (size_t)b * ldp;
        RT s = RT(0);
        for (int r = c + 1 + lane; r < m; r += 32) s = fma(pb[r], pc[r], s);
        s = warp_sum(s);
        if (lane == 0) G[b + c * w] = s + pb[c];
      }
    }
    __syncthreads();
  }
}

// T (w x w upper, ld w) of a block of w reflectors (dlarft 'F','C') from tau
// and the Gram G(b, c), b < c: T(c, c) = tau_c, T(0:c, c) = -tau_c T(0:c,
// 0:c) G(0:c, c).  One warp, lane a owns row a of T: a row depends only on
// itself, so no synchronisation between the columns.
template <typename RT = double>
__device__ void t_from_gram(const RT* G, const RT* tau, RT* T, int w) {
  const int a = threadIdx.x & 31;
  if (a >= w) return;
  for (int c = 0; c < w; c++) {
    RT v;
    if (a < c) {
      RT s = RT(0);
      for (int b = a; b < c; b++) s = fma(T[a + b * w], G[b + c * w], s);
      v = (tau[c] == RT(0)) ? RT(0) : -tau[c] * s;
    } else {
      v = (a == c) ? tau[c] : RT(0);
    }
    T[a + c * w] = v;
  }
}

// T block (dlarft 'F','C') of a w-column block whose V is stored in shared
// memory.  unit: V is unit lower (rows 0..w-1 hold the unit triangle, V(c,c)
// = 1 implicit); otherwise V is dense (TS block, top part = identity).
// G (w x w scratch) receives the needed Gram entries.  T (w x w, ld w) output.
__device__ void build_t_block(const double* V, int ldv, int m, int w, bool unit, const double* tau,
                              double* G, double* T) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int npairs = w * (w - 1) / 2;
  for (int p = warp; p < npairs; p += kWarps) {
    // decode p -> (a, c) with a < c
    int c = 1, base = 0;
    while (base + c <= p) { base += c; c++; }
    const int a = p - base;
    const double* va = V + (size_t)a * ldv;
    const double* vc = V + (size_t)c * ldv;
    double s = 0.0;
    const int r0 = unit ? c + 1 : 0;
    for (int r = r0 + lane; r < m; r += 32) s = fma(va[r], vc[r], s);
    s = warp_sum(s);
    if (lane == 0) G[a + c * w] = unit ? s + va[c] : s;
  }
  __syncthreads();
  for (int c = 0; c < w; c++) {
    const double tc = tau[c];
    const int a = threadIdx.x;
    if (a < c) {
      double s = 0.0;
      for (int b = a; b < c; b++) s = fma(T[a + b * w], G[b + c * w], s);
      T[a + c * w] = (tc == 0.0) ? 0.0 : -tc * s;
    } else if (a == c) {
      T[c + c * w] = tc;
    } else if (a < w) {
      T[a + c * w] = 0.0;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Apply the transpose of one w-column block reflector H = I - V T V^T,
// V = [Vt; Vb], to [Ct; Cb] held in shared memory:
//     W = Vt^T Ct + Vb^T Cb;  W = T^T W;  Ct -= Vt W;  Cb -= Vb W
// (notrans: H itself, W = T W).
// Vt: w x w unit lower (unit_top) or the identity; Vb: mb x w.  V and T are
// read from global memory (ld ldv / ldt).  ncol must be a multiple of 8.
// v_col0 >= 0: Vb is upper triangular (a TT merge's reflectors, stored in the
// upper triangle of a tile whose lower part holds other data): element
// (mb_off + r, c) is used when mb_off + r <= v_col0 + c, else taken as zero.
// ---------------------------------------------------------------------------
template <typename RT = double>
__device__ void apply_block_t(const double* __restrict__ gV, int ldv, int mb_off,
                              const double* __restrict__ gT, int ldt, int w, int mb, bool unit_top,
                              RT* Ct, int ldct, RT* Cb, int ldcb, int ncol, RT* smem,
                              const SmemPlan& sp, int RC, bool notrans = false, int v_col0 = -1) {
  RT* sVb = smem + sp.off_vb;
  RT* sVt = smem + sp.off_vt;
  RT* sT = smem + sp.off_t;
  RT* sW = smem + sp.off_w;
  RT* sW2 = smem + sp.off_w2;
  RT* sPart = smem + sp.off_part;
  const int tid = threadIdx.x;
  const int ldvs = RC + 1;

  // T block and the unit-lower top of V
  for (int e = tid; e < w * w; e += kThreads) {
    const int r = e % w, c = e / w;
    sT[e] = (r <= c) ? RT(ldg_cg(gT + r + (size_t)c * ldt)) : RT(0);
    if (unit_top) sVt[e] = (r > c) ? RT(ldg_cg(gV + r + (size_t)c * ldv)) : (r == c ? RT(1) : RT(0));
  }

  // ---- W = Vt^T Ct + Vb^T Cb -------------------------------------------
  const int G8 = ncol >> 3;
  const int outs = w * G8;                       // items per split
  int S = kSplitItems / (outs > 0 ? outs : 1);
  if (S < 1) S = 1;
  const int item = tid;
  const int a = item % w;
  const int g = (item / w) % (G8 > 0 ? G8 : 1);
  const int s = item / outs;
  const bool active = (outs > 0) && (item < outs * S) && (s < S);
  RT acc[8];
#pragma unroll
  for (int q = 0; q < 8; q++) acc[q] = RT(0);
  for (int r0 = 0; r0 < mb; r0 += RC) {
    const int rc = min(RC, mb - r0);
    __syncthreads();
    for (int e = tid; e < rc * w; e += kThreads) {
      const int r = e % rc, c = e / rc;
      sVb[r + c * ldvs] = (v_col0 < 0 || mb_off + r0 + r <= v_col0 + c)
                              ? RT(ldg_cg(gV + mb_off + r0 + r + (size_t)c * ldv)) : RT(0);
    }
    __syncthreads();
    if (active) {
      const RT* cb = Cb + r0 + (size_t)(8 * g) * ldcb;
      for (int r = s; r < rc; r += S) {
        const RT v = sVb[r + a * ldvs];
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] = fma(v, cb[r + (size_t)q * ldcb], acc[q]);
      }
    }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int q = 0; q < 8; q++) sPart[(s * w + a) * 8 * G8 + g * 8 + q] = acc[q];
  }
  __syncthreads();
  for (int e = tid; e < w * ncol; e += kThreads) {
    const int aa = e % w, j = e / w;
    RT v = RT(0);
    for (int ss = 0; ss < S; ss++) v += sPart[(ss * w + aa) * 8 * G8 + j];
    RT top = Ct[aa + (size_t)j * ldct];
    if (unit_top)
      for (int r = aa + 1; r < w; r++) top = fma(sVt[r + aa * w], Ct[r + (size_t)j * ldct], top);
    sW[aa + j * w] = v + top;
  }
  __syncthreads();

  // ---- W2 = T^T W (notrans: T W) --------------------------------------------
  for (int e = tid; e < w * ncol; e += kThreads) {
    const int aa = e % w, j = e / w;
    RT v = RT(0);
    if (notrans)
      for (int b = aa; b < w; b++) v = fma(sT[aa + b * w], sW[b + j * w], v);
    else
      for (int b = 0; b <= aa; b++) v = fma(sT[b + aa * w], sW[b + j * w], v);
    sW2[aa + j * w] = v;
  }
  __syncthreads();

  // ---- Ct -= Vt W2 ----------------------------------------------------------
  for (int e = tid; e < w * ncol; e += kThreads) {
    const int aa = e % w, j = e / w;
    RT v = sW2[aa + j * w];
    if (unit_top)
      for (int b = 0; b < aa; b++) v = fma(sVt[aa + b * w], sW2[b + j * w], v);
    Ct[aa + (size_t)j * ldct] -= v;
  }

  // ---- Cb -= Vb W2 ----------------------------------------------------------
  for (int r0 = 0; r0 < mb; r0 += RC) {
    const int rc = min(RC, mb - r0);
    __syncthreads();
    for (int e = tid; e < rc * w; e += kThreads) {
      const int r = e % rc, c = e / rc;
      sVb[r + c * ldvs] = (v_col0 < 0 || mb_off + r0 + r <= v_col0 + c)
                              ? RT(ldg_cg(gV + mb_off + r0 + r + (size_t)c * ldv)) : RT(0);
    }
    __syncthreads();
    for (int e = tid; e < rc * G8; e += kThreads) {
      const int r = e % rc, gg = e / rc;
      RT acc2[8];
#pragma unroll
      for (int q = 0; q < 8; q++) acc2[q] = RT(0);
      for (int b = 0; b < w; b++) {
        const RT v = sVb[r + b * ldvs];
#pragma unroll
        for (int q = 0; q < 8; q++) acc2[q] = fma(v, sW2[b + (8 * gg + q) * w], acc2[q]);
      }
      RT* cb = Cb + r0 + r + (size_t)(8 * gg) * ldcb;
#pragma unroll
      for (int q = 0; q < 8; q++) cb[(size_t)q * ldcb] -= acc2[q];
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Task bodies.  All tile pointers are global (ld = NB).  T tiles are NB x NB;
// the factorization writes their diagonal w x w blocks.
// ---------------------------------------------------------------------------

template <typename RT = double>
__device__ void load_block(RT* s, int lds, const double* g, int ldg, int m, int n) {
  for (int e = threadIdx.x; e < m * n; e += kThreads) {
    const int r = e % m, c = e / m;
    s[r + (size_t)c * lds] = RT(ldg_cg(g + r + (size_t)c * ldg));
  }
}
template <typename RT = double>
__device__ void store_block(double* g, int ldg, const RT* s, int lds, int m, int n) {
  for (int e = threadIdx.x; e < m * n; e += kThreads) {
    const int r = e % m, c = e / m;
    stg_cg(g + r + (size_t)c * ldg, double(s[r + (size_t)c * lds]));
  }
}
// The upper part (row r <= col0 + c) of an m x n block, zero below; and its
// store (a TT merge's panel columns).
template <typename RT = double>
__device__ void load_block_upper(RT* s, int lds, const double* g, int ldg, int m, int n, int col0) {
  for (int e = threadIdx.x; e < m * n; e += kThreads) {
    const int r = e % m, c = e / m;
    s[r + (size_t)c * lds] = (r <= col0 + c) ? RT(ldg_cg(g + r + (size_t)c * ldg)) : RT(0);
  }
}
template <typename RT = double>
__device__ void store_block_upper(double* g, int ldg, const RT* s, int lds, int m, int n, int col0) {
  for (int e = threadIdx.x; e < m * n; e += kThreads) {
    const int r = e % m, c = e / m;
    if (r <= col0 + c) stg_cg(g + r + (size_t)c * ldg, double(s[r + (size_t)c * lds]));
  }
}

// Points in a panel block where the DAG may act (see the executor's
// PanelPhases): after the block's reflectors are stored, before its trailing
// update, after the trailing update's first column block (first_cols wide)
// and after the whole trailing update.  These do nothing.
struct NoPanelPhases {
  __device__ int first_cols(int cb, int) const { return cb; }
  __device__ void after_panel() const {}
  __device__ void before_trailing() const {}
  __device__ void after_first() const {}
  __device__ void after_trailing() const {}
};

// Inner block b of CORE_dgeqrt(NB, NB, IB, A, NB, T, NB, TAU): the QR of
// columns [b w, (b+1) w) from row b w down (blocks 0..b-1 done), its T block,
// and its application to the columns right of it.  It writes rows >= b w of
// the tile only: rows [b w, (b+1) w) of R are final afterwards.
template <typename RT = double, class Phases = NoPanelPhases>
__device__ void task_geqrt_blk(double* A, double* T, double* tau_g, const TileShape& sh, double* smem,
                               const SmemPlan& sp, int b, const Phases& ph = Phases()) {
  const int NB = sh.NB, w = sh.w;
  RT* sm = reinterpret_cast<RT*>(smem);
  RT* sP = sm + sp.off_c1;
  RT* sTau = sm + sp.off_tau;
  RT* sG = sm + sp.off_g;
  RT* sTb = sm + sp.off_t;
  {
    const int i0 = b * w;
    const int m = NB - i0;
    __syncthreads();
    load_block(sP, NB, A + i0 + (size_t)i0 * NB, NB, m, w);
    __syncthreads();
    panel_qr_ge_fused(sP, NB, m, w, sTau, sG);
    if (threadIdx.x < 32) t_from_gram(sG, sTau, sTb, w);
    __syncthreads();
    store_block(A + i0 + (size_t)i0 * NB, NB, sP, NB, m, w);
    store_block(T + i0 + (size_t)i0 * NB, NB, sTb, w, w, w);
    for (int e = threadIdx.x; e < w; e += kThreads) stg_cg(tau_g + i0 + e, double(sTau[e]));
    __syncthreads();
    ph.after_panel();
    ph.before_trailing();
    for (int c0 = i0 + w, nc = ph.first_cols(sh.CB, w), first = 1; c0 < NB; c0 += nc, nc = sh.CB) {
      const int ncol = min(nc, NB - c0);
      RT* sC = sm + sp.off_c1;
      __syncthreads();
      load_block(sC, NB, A + i0 + (size_t)c0 * NB, NB, m, ncol);
      __syncthreads();
      apply_block_t(A + i0 + (size_t)i0 * NB, NB, w, T + i0 + (size_t)i0 * NB, NB, w, m - w, true,
                    sC, NB, sC + w, NB, ncol, sm, sp, sh.RC);
      store_block(A + i0 + (size_t)c0 * NB, NB, sC, NB, m, ncol);
      if (first) {
        first = 0;
        ph.after_first();
      }
    }
    ph.after_trailing();
  }
  __syncthreads();
}

// CORE_dgeqrt(NB, NB, IB, A, NB, T, NB, TAU)
__device__ void task_geqrt(double* A, double* T, double* tau_g, const TileShape& sh, double* smem,
                           const SmemPlan& sp) {
  for (int b = 0; b < sh.NB / sh.w; b++) task_geqrt_blk(A, T, tau_g, sh, smem, sp, b);
}

// Inner block b of CORE_dtsqrt(NB, NB, IB, A1, NB, A2, NB, T, NB, TAU): A1
// holds R (upper part) above the GEQRT's V (strict lower part, left
// untouched).  The QR of [R(bw:(b+1)w, bw:(b+1)w); A2(:, bw:(b+1)w)] (blocks
// 0..b-1 of this tile done), its T block, and its application to the columns
// right of it.  Of A1 it touches rows [b w, (b+1) w) only, and those rows are
// touched by no other block of this TSQRT: once block b is done here, block b
// of the TSQRT of the next tile below may run.
// a2_upper: the TT merge (CORE_dttqrt): A2 is upper triangular (the R of a
// domain's top tile; its strict lower part holds that tile's GEQRT reflectors
// and is neither read nor written).  The reflectors keep A2's shape, so the
// same arithmetic on A2 with zeros below the diagonal is exact, and only the
// upper triangle is stored back.
template <typename RT = double, class Phases = NoPanelPhases>
__device__ void task_tsqrt_blk(double* A1, double* A2, double* T, double* tau_g, const TileShape& sh,
                               double* smem, const SmemPlan& sp, int b, bool a2_upper = false,
                               const Phases& ph = Phases()) {
  const int NB = sh.NB, w = sh.w;
  RT* sm = reinterpret_cast<RT*>(smem);
  RT* sA = sm + sp.off_c1;     // NB x w panel of A2
  RT* sR = sm + sp.off_vt;     // w x w block of R
  RT* sTau = sm + sp.off_tau;
  RT* sG = sm + sp.off_g;
  RT* sTb = sm + sp.off_t;
  {
    const int i0 = b * w;
    __syncthreads();
    if (a2_upper)
      load_block_upper(sA, NB, A2 + (size_t)i0 * NB, NB, NB, w, i0);
    else
      load_block(sA, NB, A2 + (size_t)i0 * NB, NB, NB, w);
    load_block(sR, w, A1 + i0 + (size_t)i0 * NB, NB, w, w);
    __syncthreads();
    panel_qr_ts_fused(sR, w, sA, NB, NB, w, sTau, sG);
    if (threadIdx.x < 32) t_from_gram(sG, sTau, sTb, w);
    __syncthreads();
    if (a2_upper)
      store_block_upper(A2 + (size_t)i0 * NB, NB, sA, NB, NB, w, i0);
    else
      store_block(A2 + (size_t)i0 * NB, NB, sA, NB, NB, w);
    for (int e = threadIdx.x; e < w * w; e += kThreads) {
      const int r = e % w, c = e / w;
      if (r <= c) stg_cg(A1 + i0 + r + (size_t)(i0 + c) * NB, double(sR[r + c * w]));
    }
    store_block(T + i0 + (size_t)i0 * NB, NB, sTb, w, w, w);
    for (int e = threadIdx.x; e < w; e += kThreads) stg_cg(tau_g + i0 + e, double(sTau[e]));
    __syncthreads();
    ph.after_panel();
    ph.before_trailing();
    for (int c0 = i0 + w, nc = ph.first_cols(sh.CB, w), first = 1; c0 < NB; c0 += nc, nc = sh.CB) {
      const int ncol = min(nc, NB - c0);
      RT* sCt = sm + sp.off_c1;  // w x ncol rows of R (the panel area is free now)
      RT* sCb = sm + sp.off_c1 + w * sh.CB;  // NB x ncol of A2 after the R rows
      __syncthreads();
      // A TT merge's block reflectors reach rows < i0 + w of A2 only: the rows
      // below belong to the domain top's own later blocks, which its chain may
      // still be updating, so they are neither read nor written here.
      const int mrows = a2_upper ? i0 + w : NB;
      load_block(sCt, w, A1 + i0 + (size_t)c0 * NB, NB, w, ncol);
      load_block(sCb, NB, A2 + (size_t)c0 * NB, NB, mrows, ncol);
      __syncthreads();
      apply_block_t(A2 + (size_t)i0 * NB, NB, 0, T + i0 + (size_t)i0 * NB, NB, w, mrows, false, sCt, w,
                    sCb, NB, ncol, sm, sp, sh.RC, false, a2_upper ? i0 : -1);
      store_block(A1 + i0 + (size_t)c0 * NB, NB, sCt, w, w, ncol);
      store_block(A2 + (size_t)c0 * NB, NB, sCb, NB, mrows, ncol);
      if (first) {
        first = 0;
        ph.after_first();
      }
    }
    ph.after_trailing();
  }
  __syncthreads();
}

// CORE_dtsqrt(NB, NB, IB, A1, NB, A2, NB, T, NB, TAU)
__device__ void task_tsqrt(double* A1, double* A2, double* T, double* tau_g, const TileShape& sh,
                           double* smem, const SmemPlan& sp) {
  for (int b = 0; b < sh.NB / sh.w; b++) task_tsqrt_blk(A1, A2, T, tau_g, sh, smem, sp, b);
}

// CORE_dormqr(Left, Trans, NB, ncol, NB, IB, V, NB, T, NB, C, NB) on columns
// [c0, c0+ncol) of C (notrans: CORE_dormqr(Left, NoTrans, ...), the inner
// blocks in reverse order).
__device__ void task_larfb(const double* V, const double* T, double* C, int c0, int ncol,
                           const TileShape& sh, double* smem, const SmemPlan& sp, bool notrans = false) {
  const int NB = sh.NB, w = sh.w;
  double* sC = smem + sp.off_c1;
  __syncthreads();
  load_block(sC, NB, C + (size_t)c0 * NB, NB, NB, ncol);
  __syncthreads();
  for (int b = 0; b < NB / w; b++) {
    const int i0 = (notrans ? NB / w - 1 - b : b) * w;
    apply_block_t(V + i0 + (size_t)i0 * NB, NB, w, T + i0 + (size_t)i0 * NB, NB, w, NB - i0 - w, true,
                  sC + i0, NB, sC + i0 + w, NB, ncol, smem, sp, sh.RC, notrans);
  }
  store_block(C + (size_t)c0 * NB, NB, sC, NB, NB, ncol);
  __syncthreads();
}

// CORE_dtsmqr(Left, Trans, NB, ncol, NB, ncol, NB, IB, A1, NB, A2, NB, V, NB,
// T, NB) on columns [c0, c0+ncol) of A1 and A2 (notrans: Left, NoTrans, the
// inner blocks in reverse order).  v_upper: CORE_dttmqr, V is the upper
// triangle (with the diagonal) of its tile.
__device__ void task_ssrfb(double* A1, double* A2, const double* V, const double* T, int c0,
                           int ncol, const TileShape& sh, double* smem, const SmemPlan& sp,
                           bool notrans = false, bool v_upper = false) {
  const int NB = sh.NB, w = sh.w;
  double* s1 = smem + sp.off_c1;
  double* s2 = smem + sp.off_c2;
  __syncthreads();
  load_block(s1, NB, A1 + (size_t)c0 * NB, NB, NB, ncol);
  load_block(s2, NB, A2 + (size_t)c0 * NB, NB, NB, ncol);
  __syncthreads();
  for (int b = 0; b < NB / w; b++) {
    const int i0 = (notrans ? NB / w - 1 - b : b) * w;
    apply_block_t(V + (size_t)i0 * NB, NB, 0, T + i0 + (size_t)i0 * NB, NB, w, NB, false, s1 + i0, NB,
                  s2, NB, ncol, smem, sp, sh.RC, notrans, v_upper ? i0 : -1);
  }
  store_block(A1 + (size_t)c0 * NB, NB, s1, NB, NB, ncol);
  store_block(A2 + (size_t)c0 * NB, NB, s2, NB, NB, ncol);
  __syncthreads();
}

}  // namespace hqr
