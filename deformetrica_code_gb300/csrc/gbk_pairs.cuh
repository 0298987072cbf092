// Tiled N-body kernel template for every Gaussian kernel sum of the reference's ExactKernel
// (src/support/kernels/ExactKernel.cxx) and AbstractKernel::ConvolveSpecialHessian
// (src/support/kernels/AbstractKernel.cxx:22-88).
//
// Work decomposition. A CTA owns BLOCK*R targets (R per thread; in FP32 mode they are processed
// two at a time in float2 lanes) and one contiguous range of sources (a "split"; grid.y splits
// the source range when there are too few targets to fill 152 SMs). Sources stream through
// shared memory in tiles of TJ records, each record already converted to the lane type and
// broadcast, so the inner loop is: vector shared loads of one source record (warp-uniform
// address: a broadcast) then, per target pair, d packed subtracts, the packed r^2, one packed
// multiply for the exp argument, two MUFU ex2, and the operation's packed FMAs.
//
// Coordinates are centred per CTA: the midpoint of the CTA's target bounding box (in FP64) is
// subtracted from targets and sources before rounding to FP32, so |x - y|^2 is formed from small
// centred values (the differences themselves are never cancelled from large coordinates).
//
// Every op is linear in the source weights, so padded source slots carry zero weights and add
// exactly +0. The kernels never wait on another CTA and never use atomics: with a split, each
// split writes its own FP64 partial and a second kernel sums the splits in a fixed order, so the
// results are bitwise reproducible run to run.
#pragma once

#include <type_traits>

#include "gbk_common.cuh"

namespace gbk {

struct PairArgs {
  // targets (row-major, D columns) and optional per-target extras
  const double *x;
  long nx;
  const double *ta;  // extra A (alpha for the alpha-gradient, beta for the special Hessian)
  int ta_ld;
  const double *tb;  // extra B (xi for the special Hessian)
  int tb_ld;
  // sources (row-major, D columns), weights and optional per-source extras
  const double *y;
  long ny;
  const double *w;  // weights, pointer already offset to the first column of this chunk
  int w_ld;
  const double *sb;  // source extra B (xi for the special Hessian)
  int sb_ld;
  double sigma;
  double xscale;  // coordinates are multiplied by this before the pair loop (set by launch_pairs)
  int p0, p1, p2;  // op parameters: dim / (k, dp) / (row, col) / (k, dp, dq)
  // outputs (pointer already offset to this chunk's first column)
  double *out0;
  int out0_ld;
  double *out1;
  int out1_ld;
  int acc0, acc1;  // 1: add into out0 / out1 instead of overwriting (column chunks)
  // source split
  double *partial;  // [nsplit][NO][nx] FP64 partial sums when nsplit > 1
  long j_chunk;     // sources per split (a multiple of TJ)
  int nsplit;
  // spatial order (all null: rows in caller order, fixed target tiles, every source chunk visited)
  const int *xperm;    // sorted target position -> target row
  const int2 *xtiles;  // per CTA: [begin, end) of sorted target positions
  const int *nxtiles;  // number of valid xtiles entries
  long xtile_bound;    // grid.x for a spatial order (CTAs loop over the tiles)
  const int *yperm;    // sorted source position -> source row
  const double *ybox;  // per TJ chunk of sorted sources: lo[D], hi[D]; null = no pruning
  double prune_d2;     // a source chunk whose box is farther than this (squared) from the CTA's
                       // target box contributes exact zeros only (set by launch_pairs)
  unsigned long long *pair_count;  // if set, += (target, source) pairs this launch evaluated
  // bulk staging (lane tag f32b): 1 when y and w are the library's sorted copies, contiguous
  // (w_ld = the op's weight columns), padded to whole TJ-record chunks and 16-byte aligned, so every
  // chunk can be fetched whole by cp.async.bulk; 0 stages with ordinary loads
  int bulk;
  unsigned *status;  // device word: bit 0 set when a bounded wait of the launch gave up (null: none)
  // with nsplit > 1: one zeroed counter per target tile (index as the CTAs' tile index); the last split
  // CTA of a tile reduces the partials itself and resets it. Null: a split_reduce_kernel launch does.
  unsigned *tickets;
  // packed coordinates (caller order, small FP32 shapes; see packable): per coordinate the float pair
  // (hi, lo) of x * xscale, hi = fl32(x * xscale), lo = fl32(x * xscale - hi) (lo = 0 where hi is not
  // finite), written once per launch by pack_scaled_kernel. Null: the kernel converts a.x / a.y.
  const float2 *xp;
  const float2 *yp;
  // Fused explicit-Euler / Heun update of an output (the deformation loops; Convolve and the
  // alpha-gradients): with base0 set, the first output's element becomes
  //   out0 = base0 + aux_c0 * aux0 + step0 * v   (aux0 optional; lincomb_kernel's order of additions)
  // and, while *flag != 0 (momenta below the reference's threshold), out0 = flag_out0 (or base0 when
  // null); likewise the second output with base1 ... . base, aux and flag_out have the output's
  // layout. An output may be the launch's own targets or target extras: a CTA writes a target row
  // only after every CTA of its tile has read it (its own prologue, or the last split of the tile).
  const double *base0, *aux0, *flag_out0;
  double step0, aux_c0;
  const double *base1, *aux1, *flag_out1;
  double step1, aux_c1;
  const int *flag;
};

__device__ __forceinline__ void put(double *p, int acc, double v) {
  if (acc)
    *p += v;
  else
    *p = v;
}

// The fused update of one output element (PairArgs::base0 / base1), out of line: inlined, this rarely
// taken path changed the code generated for the whole kernel and cost the spatial-order fused pass
// about 3 % (GB300, N = M = 1e6: 546 against 531 ms per pass).
static __device__ __noinline__ void put_fused(double *out, const double *base, const double *aux, double aux_c,
                                              double step, const double *fo, const int *flag, long off, double v) {
  if (flag && *flag) {
    out[off] = fo ? fo[off] : base[off];
    return;
  }
  double r = base[off];
  if (aux) r += aux_c * aux[off];
  r += step * v;
  out[off] = r;
}

// Stores element `off` of the first (which = 0) or second output: the plain store (put) or the
// fused update of PairArgs::base0 / base1.
__device__ __forceinline__ void put_out(const PairArgs &a, int which, long off, double v) {
  double *out = which ? a.out1 : a.out0;
  const double *base = which ? a.base1 : a.base0;
  if (!base) {
    put(out + off, which ? a.acc1 : a.acc0, v);
    return;
  }
  if (which)
    put_fused(out, base, a.aux1, a.aux_c1, a.step1, a.flag_out1, a.flag, off, v);
  else
    put_fused(out, base, a.aux0, a.aux_c0, a.step0, a.flag_out0, a.flag, off, v);
}

// =============================================================================================
// Operations. Each op declares:
//   NT  : target extras (beyond x), NS : source extras (beyond y), NO : accumulators per target
//   load_target / load_source : fetch extras (FP64) for one target / one source
//   accum : per-pair update given dx = x_i - y_j, e = K_ij, target extras, source extras
//   store : final scaling of the NO FP64 sums for target i and write to the outputs
// =============================================================================================

// ExactKernel::Convolve (ExactKernel.cxx:51-74): V_i = sum_j K_ij W_j.
template <int D, int DV>
struct OpConv {
  static constexpr int NT = 0, NS = DV, NO = DV;
  __device__ static void load_target(const PairArgs &, long, double *) {}
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < DV; ++k) s[k] = a.w[j * a.w_ld + k];
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *, const SV *s, V *acc, int, int) {
    typedef Lane<T> L;
#pragma unroll
    for (int k = 0; k < DV; ++k) acc[k] = L::fma(e, s[k], acc[k]);
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
#pragma unroll
    for (int k = 0; k < DV; ++k) put_out(a, 0, i * a.out0_ld + k, v[k]);
  }
};

// Fused forward + alpha-weighted gradient: V_i = sum_j K_ij W_j (when out0 != null) and
// g_i = sum_j (alpha_i . W_j)(-2 K_ij / sigma^2)(x_i - y_j), which is
// ExactKernel::ConvolveGradient(X, alpha) (ExactKernel.cxx:264-275) and the reference CUDA
// GpuGrad1Conv1DOnDevice (lib/cuda_convolutions/GpuConv1D.cu:165-215). With CONV = false only
// the gradient is accumulated.
template <int D, int DV, bool CONV>
struct OpConvGradAlpha {
  static constexpr int NT = DV, NS = DV, NO = (CONV ? DV : 0) + D;
  __device__ static void load_target(const PairArgs &a, long i, double *t) {
#pragma unroll
    for (int k = 0; k < DV; ++k) t[k] = a.ta[i * a.ta_ld + k];
  }
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < DV; ++k) s[k] = a.w[j * a.w_ld + k];
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *t, const SV *s, V *acc, int, int) {
    typedef Lane<T> L;
    constexpr int G0 = CONV ? DV : 0;
    if (CONV) {
#pragma unroll
      for (int k = 0; k < DV; ++k) acc[k] = L::fma(e, s[k], acc[k]);
    }
    V ab = L::mul(t[0], s[0]);
#pragma unroll
    for (int k = 1; k < DV; ++k) ab = L::fma(t[k], s[k], ab);
    V c = L::mul(e, ab);
#pragma unroll
    for (int l = 0; l < D; ++l) acc[G0 + l] = L::fma(c, dx[l], acc[G0 + l]);
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
    constexpr int G0 = CONV ? DV : 0;
    if (CONV && a.out0) {
#pragma unroll
      for (int k = 0; k < DV; ++k) put_out(a, 0, i * a.out0_ld + k, v[k]);
    }
    const double f = -2.0 / (a.sigma * a.sigma * a.xscale);  // dx was accumulated pre-scaled
#pragma unroll
    for (int l = 0; l < D; ++l) put_out(a, 1, i * a.out1_ld + l, v[G0 + l] * f);
  }
};

// ExactKernel::ConvolveGradient(X) "varlin" (ExactKernel.cxx:166-202):
// G_i(k, l) = sum_j W_jk (-2 K_ij / sigma^2)(x_i - y_j)_l, output [i][k][l].
template <int D, int DV>
struct OpVarlin {
  static constexpr int NT = 0, NS = DV, NO = DV * D;
  __device__ static void load_target(const PairArgs &, long, double *) {}
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < DV; ++k) s[k] = a.w[j * a.w_ld + k];
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *, const SV *s, V *acc, int, int) {
    typedef Lane<T> L;
    V ed[D];
#pragma unroll
    for (int l = 0; l < D; ++l) ed[l] = L::mul(e, dx[l]);
#pragma unroll
    for (int k = 0; k < DV; ++k)
#pragma unroll
      for (int l = 0; l < D; ++l) acc[k * D + l] = L::fma(ed[l], s[k], acc[k * D + l]);
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
    const double f = -2.0 / (a.sigma * a.sigma * a.xscale);
#pragma unroll
    for (int o = 0; o < DV * D; ++o) put(a.out0 + i * a.out0_ld + o, a.acc0, v[o] * f);
  }
};

// ExactKernel::ConvolveGradient(X, dim) (ExactKernel.cxx:294-323): sum_j dK/dx_dim W_j, with
// dim = p0 chosen at run time (a uniform select; this op is not on the hot loop).
template <typename V>
__device__ __forceinline__ V pick(const V *v, int D, int k) {
  return k == 0 ? v[0] : (k == 1 || D < 3 ? v[1] : v[2]);
}

template <int D, int DV>
struct OpGradDim {
  static constexpr int NT = 0, NS = DV, NO = DV;
  __device__ static void load_target(const PairArgs &, long, double *) {}
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < DV; ++k) s[k] = a.w[j * a.w_ld + k];
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *, const SV *s, V *acc, int p0, int) {
    typedef Lane<T> L;
    V g = L::mul(e, pick(dx, D, p0));
#pragma unroll
    for (int k = 0; k < DV; ++k) acc[k] = L::fma(g, s[k], acc[k]);
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
    const double f = -2.0 / (a.sigma * a.sigma * a.xscale);
#pragma unroll
    for (int k = 0; k < DV; ++k) put(a.out0 + i * a.out0_ld + k, a.acc0, v[k] * f);
  }
};

// ExactKernel::ConvolveHessian(X) (ExactKernel.cxx:365-397) and its two single-entry forms
// (:399-428, :430-470). Per pair H = K (4 (x-y)(x-y)^T / sigma^4 - 2 I / sigma^2); the op keeps
// S_k(a,b) = sum_j K W_jk dx_a dx_b (a <= b) and C_k = sum_j K W_jk and forms
// H_k(a,b) = 4/sigma^4 S_k(a,b) - 2/sigma^2 delta_ab C_k at the end.
template <int D, int DV>
struct OpHessFull {
  static constexpr int NP = D * (D + 1) / 2;
  static constexpr int NT = 0, NS = DV, NO = DV * (NP + 1);
  __device__ static void load_target(const PairArgs &, long, double *) {}
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < DV; ++k) s[k] = a.w[j * a.w_ld + k];
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *, const SV *s, V *acc, int, int) {
    typedef Lane<T> L;
    V q[NP];
    int n = 0;
#pragma unroll
    for (int p = 0; p < D; ++p)
#pragma unroll
      for (int r = p; r < D; ++r) q[n++] = L::mul(dx[p], dx[r]);
#pragma unroll
    for (int k = 0; k < DV; ++k) {
      V ew = L::mul(e, s[k]);
      acc[k * (NP + 1)] = L::add(acc[k * (NP + 1)], ew);
#pragma unroll
      for (int m = 0; m < NP; ++m) acc[k * (NP + 1) + 1 + m] = L::fma(ew, q[m], acc[k * (NP + 1) + 1 + m]);
    }
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
    const double s2 = a.sigma * a.sigma;
    const double c4 = 4.0 / (s2 * s2 * a.xscale * a.xscale), c2 = 2.0 / s2;
#pragma unroll
    for (int k = 0; k < DV; ++k) {
      const double *vk = v + k * (NP + 1);
      double *o = a.out0 + i * a.out0_ld + k * D * D;
      int n = 0;
#pragma unroll
      for (int p = 0; p < D; ++p)
#pragma unroll
        for (int r = p; r < D; ++r) {
          double h = c4 * vk[1 + n++] - (p == r ? c2 * vk[0] : 0.0);
          put(o + p * D + r, a.acc0, h);
          if (r != p) put(o + r * D + p, a.acc0, h);
        }
    }
  }
};

// ExactKernel::ConvolveHessian(X, row, col) (ExactKernel.cxx:399-428) with row = p0, col = p1 at
// run time; over one weight column it is also ConvolveHessian(X, k, dp, dq) (:430-470).
// Keeps Q_k = sum_j K W_jk dx_row dx_col and C_k = sum_j K W_jk (C only matters on the diagonal).
template <int D, int DV>
struct OpHessRowCol {
  static constexpr int NT = 0, NS = DV, NO = 2 * DV;
  __device__ static void load_target(const PairArgs &, long, double *) {}
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < DV; ++k) s[k] = a.w[j * a.w_ld + k];
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *, const SV *s, V *acc, int p0, int p1) {
    typedef Lane<T> L;
    V q = L::mul(e, L::mul(pick(dx, D, p0), pick(dx, D, p1)));
#pragma unroll
    for (int k = 0; k < DV; ++k) {
      acc[2 * k] = L::fma(q, s[k], acc[2 * k]);
      acc[2 * k + 1] = L::fma(e, s[k], acc[2 * k + 1]);
    }
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
    const double s2 = a.sigma * a.sigma;
    const double c4 = 4.0 / (s2 * s2 * a.xscale * a.xscale), c2 = 2.0 / s2;
#pragma unroll
    for (int k = 0; k < DV; ++k) {
      double h = c4 * v[2 * k] - (a.p0 == a.p1 ? c2 * v[2 * k + 1] : 0.0);
      put(a.out0 + i * a.out0_ld + k, a.acc0, h);
    }
  }
};

// Fused ConvolveSpecialHessian (AbstractKernel.cxx:22-88; reference CUDA GradDiff,
// GpuConv1D.cu:552-607 scaled by -1/2 at CUDAExactKernel.cxx:223) over the sources themselves:
// gamma_i = sum_j (beta_i . beta_j) H_ij (xi_j - xi_i)
//         = sum_j (b.b) K [4/sigma^4 ((y_i - y_j).(xi_j - xi_i)) (y_i - y_j) - 2/sigma^2 (xi_j - xi_i)].
// Targets carry (y_i, beta_i, xi_i), sources (y_j, beta_j, xi_j).
template <int D>
struct OpSpecialHessian {
  static constexpr int NT = 2 * D, NS = 2 * D, NO = 2 * D;
  __device__ static void load_target(const PairArgs &a, long i, double *t) {
#pragma unroll
    for (int k = 0; k < D; ++k) t[k] = a.ta[i * a.ta_ld + k];
#pragma unroll
    for (int k = 0; k < D; ++k) t[D + k] = -a.tb[i * a.tb_ld + k];  // -xi_i
  }
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < D; ++k) s[k] = a.w[j * a.w_ld + k];
#pragma unroll
    for (int k = 0; k < D; ++k) s[D + k] = a.sb[j * a.sb_ld + k];
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *t, const SV *s, V *acc, int, int) {
    typedef Lane<T> L;
    V bb = L::mul(t[0], s[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) bb = L::fma(t[k], s[k], bb);
    V de[D];
#pragma unroll
    for (int k = 0; k < D; ++k) de[k] = L::add(s[D + k], t[D + k]);  // xi_j - xi_i
    V q = L::mul(dx[0], de[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) q = L::fma(dx[k], de[k], q);
    V c = L::mul(e, bb);
    V cq = L::mul(c, q);
#pragma unroll
    for (int k = 0; k < D; ++k) {
      acc[k] = L::fma(cq, dx[k], acc[k]);
      acc[D + k] = L::fma(c, de[k], acc[D + k]);
    }
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
    const double s2 = a.sigma * a.sigma;
    const double c4 = 4.0 / (s2 * s2 * a.xscale * a.xscale), c2 = 2.0 / s2;
#pragma unroll
    for (int k = 0; k < D; ++k) put(a.out0 + i * a.out0_ld + k, a.acc0, c4 * v[k] - c2 * v[D + k]);
  }
};

// The control-point part of AdjointEquationsIntegrator::ComputeUpdateAt
// (AdjointEquationsIntegrator.cxx:476-570) in ONE pass over the CP x CP pairs. The reference
// makes five kernel calls for it (Convolve and varlin ConvolveGradient of [p | xi_pos], d calls of
// ConvolveGradient(X, dim) with weights xi_mom[:, dim] p, and ConvolveSpecialHessian(xi_mom));
// with dx = x_i - x_j, dK = -2 K dx / sigma^2, dxi = xi_mom_j - xi_mom_i they sum to
//   dXi3_i = sum_j (xi_pos_i . p_j + p_i . xi_pos_j) dK
//   dXi4_i = sum_j (p_i . p_j) K [4/sigma^4 (dx . dxi) dx - 2/sigma^2 dxi]
//   dXi5_i = sum_j K xi_pos_j
//   dXi6_i = sum_j (dK . dxi) p_j
// and the op writes dPos = dXi3 + dXi4 (out0) and dMom = dXi5 + dXi6 (out1).
// Target and source extras are (p, xi_pos, xi_mom): ta -> p, tb -> xi_pos, a.sb -> xi_mom, all
// with leading dimension D.
template <int D>
struct OpAdjointCP {
  static constexpr int NT = 3 * D, NS = 3 * D, NO = 5 * D;
  __device__ static void load_target(const PairArgs &a, long i, double *t) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      t[k] = a.ta[i * D + k];
      t[D + k] = a.tb[i * D + k];
      t[2 * D + k] = -a.sb[i * D + k];  // -xi_mom_i
    }
  }
  __device__ static void load_source(const PairArgs &a, long j, double *s) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      s[k] = a.w[j * D + k];
      s[D + k] = a.tb[j * D + k];
      s[2 * D + k] = a.sb[j * D + k];
    }
  }
  template <typename T, typename V, typename SV>
  __device__ __forceinline__ static void accum(const V *dx, V e, const V *t, const SV *s, V *acc, int, int) {
    typedef Lane<T> L;
    // t: p_i, xp_i, -xm_i ; s: p_j, xp_j, xm_j
    V a1 = L::mul(t[D], s[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) a1 = L::fma(t[D + k], s[k], a1);
#pragma unroll
    for (int k = 0; k < D; ++k) a1 = L::fma(t[k], s[D + k], a1);
    V bb = L::mul(t[0], s[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) bb = L::fma(t[k], s[k], bb);
    V dxi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) dxi[k] = L::add(s[2 * D + k], t[2 * D + k]);
    V q = L::mul(dx[0], dxi[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) q = L::fma(dx[k], dxi[k], q);
    V ka = L::mul(e, a1), kb = L::mul(e, bb);
    V kbq = L::mul(kb, q), kq = L::mul(e, q);
#pragma unroll
    for (int k = 0; k < D; ++k) {
      acc[k] = L::fma(ka, dx[k], acc[k]);                  // A
      acc[D + k] = L::fma(kbq, dx[k], acc[D + k]);         // B
      acc[2 * D + k] = L::fma(kb, dxi[k], acc[2 * D + k]); // C
      acc[3 * D + k] = L::fma(e, s[D + k], acc[3 * D + k]);  // E
      acc[4 * D + k] = L::fma(kq, s[k], acc[4 * D + k]);   // F
    }
  }
  __device__ static void store(const PairArgs &a, long i, const double *v) {
    const double s2 = a.sigma * a.sigma, xs = a.xscale;
    const double cg = -2.0 / (s2 * xs), c4 = 4.0 / (s2 * s2 * xs * xs), c2 = -2.0 / s2;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      put(a.out0 + i * a.out0_ld + k, a.acc0, cg * v[k] + c4 * v[D + k] + c2 * v[2 * D + k]);
      put(a.out1 + i * a.out1_ld + k, a.acc1, v[3 * D + k] + cg * v[4 * D + k]);
    }
  }
};

// =============================================================================================
// The kernel.
// =============================================================================================
template <typename T>
struct SrcLane;
template <>
struct SrcLane<float> {
  typedef float2 SV;
};
template <>
struct SrcLane<f32w> {
  typedef float2 SV;
};
template <>
struct SrcLane<f32b> {
  typedef float2 SV;
};
template <>
struct SrcLane<f32s> {
  typedef float SV;
};
template <>
struct SrcLane<double> {
  typedef double SV;
};

// Packs the values of the W targets of one lane group (FP32: two targets, FP64: one).
template <typename T>
struct Pack;
template <>
struct Pack<float> {
  __device__ __forceinline__ static float2 make(double a, double b) { return make_float2((float)a, (float)b); }
  __device__ __forceinline__ static float2 make(float a, float b) { return make_float2(a, b); }
};
template <>
struct Pack<f32w> : Pack<float> {};
template <>
struct Pack<f32b> : Pack<float> {};
template <>
struct Pack<f32s> {
  __device__ __forceinline__ static float make(double a, double) { return (float)a; }
  __device__ __forceinline__ static float make(float a, float) { return a; }
};
template <>
struct Pack<double> {
  __device__ __forceinline__ static double make(double a, double) { return a; }
};

// Launch shapes that read packed coordinates (PairArgs::xp / yp) in caller order: the small FP32 shapes.
// Their CTAs own few targets and short source ranges, so converting coordinates from FP64 in every
// CTA (the bounding box, the centring and the scaling, repeated for every target tile and source
// split) costs more than their pair work on a GPU whose FP64 rate is ~1/64 of FP32; with packed
// coordinates a CTA centres in FP32 only.
template <typename T, int BLOCK>
__host__ __device__ constexpr bool packable() {
  return BLOCK <= 64 && (std::is_same<T, float>::value || std::is_same<T, f32w>::value ||
                         std::is_same<T, f32s>::value);
}

// The centred coordinate q = p - c of a packed coordinate p = hi + lo and a float centre c, in FP32:
// hi - c exactly as a + e (Knuth's TwoSum), then qh = fl(a + fl(e + lo)) -- q rounded once up to the
// rounding of the small term -- and ql = fl((a - qh) + fl(e + lo)), the low part for two-float
// coordinates (qh + ql = q to ~2^-48 |q|).
__device__ __forceinline__ void centre_packed(float2 p, float c, float &qh, float &ql) {
  const float a = __fsub_rn(p.x, c);
  const float bb = __fsub_rn(a, p.x);
  const float e = __fadd_rn(__fsub_rn(p.x, __fsub_rn(a, bb)), __fsub_rn(-c, bb));
  const float t = __fadd_rn(e, p.y);
  qh = __fadd_rn(a, t);
  ql = __fadd_rn(__fsub_rn(a, qh), t);
}

// Source record: D coordinates, the op's NS extras and, for two-float coordinates, the D low
// parts; padded so that a record is a whole number of 16-byte vectors.
template <class Op, int D, typename T>
struct Rec {
  static constexpr int LO = D + Op::NS;  // first low part (two-float coordinates only)
  static constexpr int NJ = D + Op::NS + (std::is_same<T, f32w>::value ? D : 0);
  static constexpr int PER16 = 16 / (int)sizeof(typename SrcLane<T>::SV);
  static constexpr int NJP = (NJ + PER16 - 1) / PER16 * PER16;
};

// Dynamic shared memory of one CTA: the source tile, then (CSM > 0) the per-thread compensation
// terms (CSM = 1) or running sums and compensation terms (CSM = 2) of the G lane groups.
template <class Op, typename T, int D, int BLOCK, int R, int TJ, int CSM>
constexpr size_t pair_smem_bytes() {
  return (size_t)TJ * Rec<Op, D, T>::NJP * sizeof(typename SrcLane<T>::SV) +
         (size_t)CSM * (R / Lane<T>::kWidth) * Op::NO * BLOCK * sizeof(typename Lane<T>::V) +
         (std::is_same<T, f32b>::value ? (size_t)2 * TJ * (D + Op::NS) * sizeof(double) : 0);
}

// Bulk staging state of a CTA (lane tag f32b): the two buffers' mbarriers, the parity each waits for
// next, and the elected thread's verdict on the last wait. One instance per kernel, kept across the
// target tiles a CTA loops over.
struct BulkState {
  unsigned long long bar[2];
  unsigned parity[2];
  unsigned ok;
};
__device__ __forceinline__ BulkState &bulk_state() {
  __shared__ BulkState s;
  return s;
}
// Called by every thread of a bulk-staging kernel before its first tile.
__device__ __forceinline__ void bulk_init() {
  BulkState &st = bulk_state();
  if (threadIdx.x == 0) {
    mbar_init(&st.bar[0], 1);
    mbar_init(&st.bar[1], 1);
    st.parity[0] = st.parity[1] = 0;
    st.ok = 1;
    mbar_fence_init();
  }
  __syncthreads();
}

// Source chunks per visit mask (pruning): 512 bytes of shared memory.
constexpr int kPruneWindow = 4096;
// Adaptive two-float coordinates (lane tag f32w): a CTA whose target box is wider than this, in units
// of the FP32 coordinate scale, uses hi + lo coordinates; the spatial order's tiles never are.
constexpr double kTwoFloatWidth = 16.0;

// The pair loop of one CTA after its targets and centre are known: stage each source tile, evaluate
// every (target, source) pair, fold the compensated sums, write the results. TWOF: two-float
// coordinates (hi + lo parts of targets and staged sources); the record stride follows TWOF, so the
// one-float loop of an adaptive kernel reads no low parts.
template <class Op, typename T, int D, int BLOCK, int R, int TJ, int MERGE, int UNR, int CSM, bool TWOF>
__device__ __forceinline__ void pair_body(const PairArgs &a, const long tile_idx, const int split, const long i0,
                                          const long iend,
                                          const double *ctr, const float *ctrf, const double *s_box,
                                          unsigned *s_visit, unsigned char *smem_raw) {
  typedef Lane<T> L;
  typedef typename L::V V;
  typedef typename SrcLane<T>::SV SV;
  constexpr int W = L::kWidth;
  constexpr int G = R / W;
  constexpr int LO = D + Op::NS;  // first low part of a record (TWOF)
  constexpr int NJ = D + Op::NS + (TWOF ? D : 0);
  constexpr int PER16 = 16 / (int)sizeof(SV);
  constexpr int NJP = (NJ + PER16 - 1) / PER16 * PER16;
  constexpr int NO = Op::NO;
  static_assert(NJP <= Rec<Op, D, T>::NJP, "the tile is sized for the widest record");
  SV *tile = reinterpret_cast<SV *>(smem_raw);
  const int *const xperm = a.xperm;
  const int *const yperm = a.yperm;
  const bool prune = a.ybox != nullptr;
  const double xs = a.xscale;
  constexpr bool PK = packable<T, BLOCK>();
  const bool packed = PK && a.xp != nullptr;  // caller order: no permutation, no pruning
  // ---- this thread's targets: centred, pre-scaled coordinates and extras, in lanes ----
  V xg[G][D];
  V xlo[G][TWOF ? D : 1];  // low parts of two-float coordinates
  V tg[G][Op::NT > 0 ? Op::NT : 1];
  if constexpr (PK) {
    if (packed) {
#pragma unroll
      for (int g = 0; g < G; ++g) {
        float qh[W][D], ql[W][D];
        double tv[W][Op::NT > 0 ? Op::NT : 1];
#pragma unroll
        for (int w2 = 0; w2 < W; ++w2) {
          long i = i0 + threadIdx.x + (long)(g * W + w2) * BLOCK;
          // out-of-range lanes compute a copy, never stored
          const long ic = checked_index(i < iend ? i : (iend - 1), a.nx, a.status);
#pragma unroll
          for (int l = 0; l < D; ++l) centre_packed(a.xp[ic * D + l], ctrf[l], qh[w2][l], ql[w2][l]);
          Op::load_target(a, ic, tv[w2]);
        }
#pragma unroll
        for (int l = 0; l < D; ++l) {
          xg[g][l] = Pack<T>::make(qh[0][l], qh[W - 1][l]);
          if (TWOF) xlo[g][l < (TWOF ? D : 1) ? l : 0] = Pack<T>::make(ql[0][l], ql[W - 1][l]);
        }
#pragma unroll
        for (int k = 0; k < Op::NT; ++k) tg[g][k] = Pack<T>::make(tv[0][k], tv[W - 1][k]);
      }
    }
  }
#pragma unroll
  for (int g = 0; g < G; ++g) {
    if (packed) break;
    double xv[W][D], tv[W][Op::NT > 0 ? Op::NT : 1];
#pragma unroll
    for (int w2 = 0; w2 < W; ++w2) {
      long i = i0 + threadIdx.x + (long)(g * W + w2) * BLOCK;
      long ic = checked_index(i < iend ? i : (iend - 1), a.nx, a.status);  // out-of-range lanes: a copy
      if (xperm) ic = checked_index(xperm[ic], a.nx, a.status);
#pragma unroll
      for (int l = 0; l < D; ++l) xv[w2][l] = (a.x[ic * D + l] - ctr[l]) * xs;
      Op::load_target(a, ic, tv[w2]);
    }
#pragma unroll
    for (int l = 0; l < D; ++l) xg[g][l] = Pack<T>::make(xv[0][l], xv[W - 1][l]);
    if (TWOF) {
#pragma unroll
      for (int l = 0; l < D; ++l) {
        const double h0 = (double)(float)xv[0][l], h1 = (double)(float)xv[W - 1][l];
        xlo[g][l < (TWOF ? D : 1) ? l : 0] = Pack<T>::make(xv[0][l] - h0, xv[W - 1][l] - h1);
      }
    }
#pragma unroll
    for (int k = 0; k < Op::NT; ++k) tg[g][k] = Pack<T>::make(tv[0][k], tv[W - 1][k]);
  }

  // running sums / compensation: registers, or shared memory after the tile (CSM)
  V *csm = reinterpret_cast<V *>(smem_raw + (size_t)TJ * Rec<Op, D, T>::NJP * sizeof(SV));
  V acc[G][NO], sum[G][NO], cmp[G][NO];
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int o = 0; o < NO; ++o) {
      acc[g][o] = L::zero();
      sum[g][o] = L::zero();
      cmp[g][o] = L::zero();
      if (CSM >= 1) csm[(g * NO + o) * BLOCK + threadIdx.x] = L::zero();
      if (CSM >= 2) csm[((G + g) * NO + o) * BLOCK + threadIdx.x] = L::zero();
    }

  const V cx = exp_arg_scale<T>(a.sigma);
  const int p0 = a.p0, p1 = a.p1;

  const long jb = (long)split * a.j_chunk;
  long je = jb + a.j_chunk;
  if (je > a.ny) je = a.ny;
  long visited = 0;  // sources of the visited chunks

  // Visit mask of the kPruneWindow source chunks from jt: one distance test per chunk for the whole
  // CTA (FP64, spread over the threads), then one shared-memory bit per chunk. Collective.
  auto make_mask = [&](const long jt) {
    __syncthreads();  // every thread is done with the previous window's mask
#pragma unroll 4
    for (int r = 0; r < kPruneWindow / BLOCK; ++r) {
      const long jc = jt + (long)(r * BLOCK + threadIdx.x) * TJ;  // first source of the chunk
      bool visit = false;
      if (jc < je) {
        const double *cb = a.ybox + (jc / TJ) * (2 * D);
        double d2 = 0.0;
#pragma unroll
        for (int l = 0; l < D; ++l) {
          const double gap = fmax(0.0, fmax(cb[l] - s_box[D + l], s_box[l] - cb[D + l]));
          d2 += gap * gap;
        }
        visit = !(d2 > a.prune_d2);
      }
      const unsigned bits = __ballot_sync(0xffffffffu, visit);
      if ((threadIdx.x & 31) == 0) s_visit[(r * BLOCK + threadIdx.x) >> 5] = bits;
    }
    __syncthreads();
  };

  // Every pair of the staged tile's first cnt sources with the thread's targets, folded into the
  // compensated sums run by run.
  auto compute_tile = [&](const int cnt) {
    const int nrun = (cnt + MERGE - 1) / MERGE;
    for (int run = 0; run < nrun; ++run) {
      const SV *rp = tile + run * MERGE * NJP;
#pragma unroll UNR
      for (int jj = 0; jj < MERGE; ++jj) {
        SV s[NJP];
        const float4 *src = reinterpret_cast<const float4 *>(rp + jj * NJP);
#pragma unroll
        for (int q = 0; q < (int)(NJP * sizeof(SV) / 16); ++q) {
          float4 v4 = src[q];
          *reinterpret_cast<float4 *>(reinterpret_cast<char *>(s) + 16 * q) = v4;
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
          V dx[D];
#pragma unroll
          for (int l = 0; l < D; ++l) dx[l] = L::add(xg[g][l], s[l]);
          if (TWOF) {  // (x_hi - y_hi) + (x_lo - y_lo); the staged source values are negated
#pragma unroll
            for (int l = 0; l < D; ++l) dx[l] = L::add(dx[l], L::add(xlo[g][l < (TWOF ? D : 1) ? l : 0], s[LO + l]));
          }
          V r2 = L::mul(dx[0], dx[0]);
#pragma unroll
          for (int l = 1; l < D; ++l) r2 = L::fma(dx[l], dx[l], r2);
          V e = L::kexp(r2, cx);
          Op::template accum<T>(dx, e, tg[g], s + D, acc[g], p0, p1);
        }
      }
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int o = 0; o < NO; ++o) {
          if (CSM == 0) {
            Comp<T>::fold(sum[g][o], cmp[g][o], acc[g][o]);
          } else {
            V &cm = csm[(g * NO + o) * BLOCK + threadIdx.x];
            V c = cm;
            if (CSM == 1) {
              Comp<T>::fold(sum[g][o], c, acc[g][o]);
            } else {
              V &sm = csm[((G + g) * NO + o) * BLOCK + threadIdx.x];
              V s2 = sm;
              Comp<T>::fold(s2, c, acc[g][o]);
              sm = s2;
            }
            cm = c;
          }
          acc[g][o] = L::zero();
        }
    }
  };

  if constexpr (std::is_same<T, f32b>::value) {
    if (a.bulk) {  // bulk asynchronous staging of the library's chunk-padded sorted source copies
      static_assert(!TWOF && NJ == D + Op::NS, "bulk staging stages coordinates and weights only");
      BulkState &st = bulk_state();
      double *raw = reinterpret_cast<double *>(smem_raw + (size_t)TJ * Rec<Op, D, T>::NJP * sizeof(SV) +
                                               (size_t)CSM * G * NO * BLOCK * sizeof(V));
      constexpr unsigned kBytesY = TJ * D * sizeof(double), kBytesW = TJ * Op::NS * sizeof(double);
      const long nch = (je - jb + TJ - 1) / TJ;  // chunks of this split
      long cur_window = -1;
      // first visited chunk >= q of this split, or nch (collective: may build a window's mask)
      auto next_visited = [&](long q) -> long {
        while (q < nch) {
          if (!prune) return q;
          const long wbase = q - q % kPruneWindow;
          if (wbase != cur_window) {
            make_mask(jb + wbase * TJ);
            cur_window = wbase;
          }
          const int wq = (int)(q - wbase);
          for (int w = wq >> 5; w < kPruneWindow / 32; ++w) {
            unsigned bits = s_visit[w];
            if (w == (wq >> 5)) bits &= ~0u << (wq & 31);
            if (bits) {
              const long c = wbase + w * 32 + (__ffs(bits) - 1);
              return c < nch ? c : nch;
            }
          }
          q = wbase + kPruneWindow;
        }
        return nch;
      };
      // the elected thread fetches chunk q (coordinates, then weights) into buffer b
      auto issue = [&](const long q, const int b) {
        double *ry = raw + (size_t)b * TJ * (D + Op::NS);
        const long jt = checked_index(jb + q * TJ, a.ny, a.status);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&st.bar[b], kBytesY + kBytesW);
        bulk_copy_g2s(ry, a.y + jt * D, kBytesY, &st.bar[b]);
        bulk_copy_g2s(ry + TJ * D, a.w + jt * Op::NS, kBytesW, &st.bar[b]);
      };
      unsigned par[2] = {st.parity[0], st.parity[1]};
      long q = next_visited(0);
      int b = 0;
      if (threadIdx.x == 0 && q < nch) issue(q, 0);
      while (q < nch) {
        const long jt = jb + q * TJ;
        const int cnt = (int)((je - jt) < TJ ? (je - jt) : TJ);
        visited += cnt;
        if (threadIdx.x == 0) st.ok = mbar_wait_bounded(&st.bar[b], par[b]) ? 1u : 0u;
        __syncthreads();
        if (!st.ok) {  // the copy never completed: report it; the CTA stops (pair_kernel checks st.ok)
          if (threadIdx.x == 0 && a.status) atomicOr(a.status, 1u);
          return;
        }
        par[b] ^= 1u;
        const double *ry = raw + (size_t)b * TJ * (D + Op::NS), *rw = ry + TJ * D;
        for (int r = threadIdx.x; r < TJ; r += BLOCK) {
          double rec[NJP];
#pragma unroll
          for (int l = 0; l < D; ++l) rec[l] = r < cnt ? (ctr[l] - ry[r * D + l]) * xs : 0.0;
#pragma unroll
          for (int k = 0; k < Op::NS; ++k) rec[D + k] = r < cnt ? rw[r * Op::NS + k] : 0.0;
#pragma unroll
          for (int k = NJ; k < NJP; ++k) rec[k] = 0.0;
#pragma unroll
          for (int k = 0; k < NJP; ++k) tile[r * NJP + k] = SrcVal<T>::make(rec[k]);
        }
        const long nq = next_visited(q + 1);
        __syncthreads();  // the tile is staged and buffer b consumed
        if (threadIdx.x == 0 && nq < nch) issue(nq, b ^ 1);  // overlaps the tile's pair work
        compute_tile(cnt);
        __syncthreads();
        q = nq;
        b ^= 1;
      }
      if (threadIdx.x == 0) {
        st.parity[0] = par[0];
        st.parity[1] = par[1];
      }
      goto sums_done;
    }
  }

  for (long jt = jb; jt < je; jt += TJ) {
    if (prune) {
      const long q = (jt - jb) / TJ;
      const int wq = (int)(q % kPruneWindow);
      if (wq == 0) make_mask(jt);
      if (!((s_visit[wq >> 5] >> (wq & 31)) & 1u)) continue;  // same decision in every thread
    }
    const int cnt = (int)((je - jt) < TJ ? (je - jt) : TJ);
    visited += cnt;
    if constexpr (PK) {
      if (packed) {  // -(y' - c) from the packed coordinates in FP32, extras converted from FP64
        for (int r = threadIdx.x; r < TJ; r += BLOCK) {
          SV rv[NJP];
#pragma unroll
          for (int q = 0; q < NJP; ++q) rv[q] = SrcVal<T>::make(0.f);  // padding and empty slots: exact no-ops
          if (r < cnt) {
            const long j = checked_index(jt + r, a.ny, a.status);
            double ex[Op::NS > 0 ? Op::NS : 1];
            Op::load_source(a, j, ex);
#pragma unroll
            for (int l = 0; l < D; ++l) {
              float qh, ql;
              centre_packed(a.yp[j * D + l], ctrf[l], qh, ql);
              rv[l] = SrcVal<T>::make(-qh);
              if (TWOF) rv[LO + l < NJP ? LO + l : 0] = SrcVal<T>::make(-ql);
            }
#pragma unroll
            for (int k = 0; k < Op::NS; ++k) rv[D + k] = SrcVal<T>::make(ex[k]);
          }
#pragma unroll
          for (int q = 0; q < NJP; ++q) tile[r * NJP + q] = rv[q];
        }
        __syncthreads();
        compute_tile(cnt);
        __syncthreads();
        continue;
      }
    }
    // ---- stage TJ source records: -(y - c) * xscale and extras, broadcast to the lane type ----
    for (int r = threadIdx.x; r < TJ; r += BLOCK) {
      double rec[NJP];
      if (r < cnt) {
        long j = checked_index(jt + r, a.ny, a.status);
        if (yperm) j = checked_index(yperm[j], a.ny, a.status);
#pragma unroll
        for (int l = 0; l < D; ++l) rec[l] = (ctr[l] - a.y[j * D + l]) * xs;
        Op::load_source(a, j, rec + D);
        if (TWOF) {
#pragma unroll
          for (int l = 0; l < D; ++l) rec[LO + l] = rec[l] - (double)(float)rec[l];
        }
      } else {
#pragma unroll
        for (int q = 0; q < NJ; ++q) rec[q] = 0.0;  // zero weights: exact no-op
      }
#pragma unroll
      for (int q = NJ; q < NJP; ++q) rec[q] = 0.0;
#pragma unroll
      for (int q = 0; q < NJP; ++q) tile[r * NJP + q] = SrcVal<T>::make(rec[q]);
    }
    __syncthreads();

    compute_tile(cnt);
    __syncthreads();
  }

sums_done:
  if (a.pair_count && threadIdx.x == 0 && visited > 0)
    atomicAdd(a.pair_count, (unsigned long long)(iend - i0) * (unsigned long long)visited);

  // ---- write: final sums in FP64 ----
#pragma unroll
  for (int g = 0; g < G; ++g) {
#pragma unroll
    for (int w2 = 0; w2 < W; ++w2) {
      long i = i0 + threadIdx.x + (long)(g * W + w2) * BLOCK;
      if (i >= iend) continue;
      double v[NO];
#pragma unroll
      for (int o = 0; o < NO; ++o) {
        V sv = CSM >= 2 ? csm[((G + g) * NO + o) * BLOCK + threadIdx.x] : sum[g][o];
        V cv = CSM >= 1 ? csm[(g * NO + o) * BLOCK + threadIdx.x] : cmp[g][o];
        v[o] = (double)L::get(sv, w2) + (double)L::get(cv, w2);
      }
      if (a.nsplit > 1) {  // partials by sorted position; the reduction maps to rows
        double *p = a.partial + (long)split * NO * a.nx;
#pragma unroll
        for (int o = 0; o < NO; ++o) p[(long)o * a.nx + i] = v[o];
      } else {
        Op::store(a, checked_index(xperm ? (long)xperm[i] : i, a.nx, a.status), v);
      }
    }
  }
  if (a.nsplit > 1 && a.tickets) {
    // Fused split reduction: the last of the tile's nsplit CTAs to finish (a ticket per tile, counted
    // with one atomic per CTA after its partials are fenced) sums the partials in split order, as
    // split_reduce_kernel does, and resets the ticket for the next launch. No CTA waits for another.
    __shared__ unsigned s_last;
    __syncthreads();  // every thread's partials are written
    if (threadIdx.x == 0) {
      __threadfence();
      s_last = atomicAdd(a.tickets + tile_idx, 1u) == (unsigned)(a.nsplit - 1);
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      // SB splits' partials are loaded before they are added (in split order, as the separate
      // reduction adds them), so a CTA waits for one round of L2 loads per SB splits, not per split.
      constexpr int SB_VALS = BLOCK <= 64 ? 24 : 12;  // small shapes have registers to spare here
      constexpr int SB = NO >= SB_VALS ? 1 : SB_VALS / NO;
      for (int r = 0; r < R; ++r) {
        const long i = i0 + threadIdx.x + (long)r * BLOCK;
        if (i >= iend) continue;
        double v[NO];
#pragma unroll
        for (int o = 0; o < NO; ++o) v[o] = 0.0;
        for (int s0 = 0; s0 < a.nsplit; s0 += SB) {
          double buf[SB][NO];
#pragma unroll
          for (int k = 0; k < SB; ++k) {
            const double *p = a.partial + (long)(s0 + k < a.nsplit ? s0 + k : s0) * NO * a.nx;
#pragma unroll
            for (int o = 0; o < NO; ++o) buf[k][o] = __ldcg(p + (long)o * a.nx + i);
          }
#pragma unroll
          for (int k = 0; k < SB; ++k)
            if (s0 + k < a.nsplit) {
#pragma unroll
              for (int o = 0; o < NO; ++o) v[o] += buf[k][o];
            }
        }
        Op::store(a, checked_index(xperm ? (long)xperm[i] : i, a.nx, a.status), v);
      }
      if (threadIdx.x == 0) a.tickets[tile_idx] = 0u;
    }
  }
}

// FP32 mode subtracts the CTA's target bounding-box midpoint (centring); FP64 mode forms x - y
// directly, as the reference does. UNR: unroll of the per-source loop. CSM: see pair_smem_bytes.
// With a spatial order (a.xtiles), the CTA's targets are the sorted positions of its tile, rows
// a.xperm[...]; sources are visited in sorted order (a.yperm) and a source chunk whose box is
// farther than a.prune_d2 from the CTA's target box is skipped: every pair term in it is exactly
// zero, so the sums are the same as when it is visited.
template <class Op, typename T, int D, int BLOCK, int R, int TJ, int MERGE, int UNR, int CSM>
__device__ __forceinline__ void pair_block(const PairArgs &a, const long tile_idx, const int split) {
  constexpr bool CENTER = !std::is_same<T, double>::value;
  static_assert(R % Lane<T>::kWidth == 0, "R must be a multiple of the lane width");
  static_assert(TJ % MERGE == 0, "TJ must be a multiple of MERGE");
  static_assert(BLOCK % 32 == 0 && kPruneWindow % BLOCK == 0, "visit-mask rounds need whole warps");

  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_red[2 * D][BLOCK / 32];
  __shared__ double s_ctr[D];
  __shared__ double s_box[2 * D];
  __shared__ unsigned s_visit[kPruneWindow / 32];
  constexpr bool PK = packable<T, BLOCK>();
  __shared__ float s_redf[PK ? 2 * D : 1][BLOCK / 32];
  __shared__ float s_ctrf[D];
  __shared__ float s_widf;

  // ---- this CTA's targets: sorted positions [i0, iend) (caller order when unsorted) ----
  long i0, iend;
  if (a.xtiles) {
    if (tile_idx >= (long)*a.nxtiles) return;  // beyond the tiles of this order: whole CTA
    const int2 tl = a.xtiles[tile_idx];
    i0 = tl.x;
    iend = tl.y;
  } else {
    i0 = tile_idx * (BLOCK * R);
    iend = i0 + BLOCK * R < a.nx ? i0 + BLOCK * R : a.nx;
  }
  const int *const xperm = a.xperm;
  const bool prune = a.ybox != nullptr;
  const bool packed = PK && a.xp != nullptr;

  // ---- bounding box of the CTA's targets (FP64): centre for FP32 lanes, box for pruning ----
  double ctr[D];
  float ctrf[D];
  if constexpr (PK) {
    if (packed) {
      // Packed coordinates (caller order, no pruning): the box of the high parts in FP32 (scaled units),
      // its midpoint as the CTA's float centre; NaN coordinates are ignored by fminf / fmaxf.
      float lo[D], hi[D];
#pragma unroll
      for (int l = 0; l < D; ++l) {
        lo[l] = 3.0e38f;
        hi[l] = -3.0e38f;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const long i = i0 + threadIdx.x + (long)r * BLOCK;
        if (i < iend) {
#pragma unroll
          for (int l = 0; l < D; ++l) {
            const float v = a.xp[checked_index(i, a.nx, a.status) * D + l].x;
            lo[l] = fminf(lo[l], v);
            hi[l] = fmaxf(hi[l], v);
          }
        }
      }
#pragma unroll
      for (int l = 0; l < D; ++l) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          lo[l] = fminf(lo[l], __shfl_xor_sync(0xffffffffu, lo[l], o));
          hi[l] = fmaxf(hi[l], __shfl_xor_sync(0xffffffffu, hi[l], o));
        }
      }
      if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int l = 0; l < D; ++l) {
          s_redf[l][threadIdx.x >> 5] = lo[l];
          s_redf[D + l][threadIdx.x >> 5] = hi[l];
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        float wid = 0.f;
        for (int l = 0; l < D; ++l) {
          float mn = 3.0e38f, mx = -3.0e38f;
          for (int w2 = 0; w2 < BLOCK / 32; ++w2) {
            mn = fminf(mn, s_redf[l][w2]);
            mx = fmaxf(mx, s_redf[D + l][w2]);
          }
          s_ctrf[l] = mn <= mx ? 0.5f * mn + 0.5f * mx : 0.f;
          wid = fmaxf(wid, mx - mn);  // an infinite spread makes the CTA wide, as the FP64 box does
        }
        s_widf = wid;
      }
      __syncthreads();
#pragma unroll
      for (int l = 0; l < D; ++l) {
        ctrf[l] = s_ctrf[l];
        ctr[l] = 0.0;
      }
    }
  }
  if (packed) {
  } else if (CENTER || prune) {
    double lo[D], hi[D];
#pragma unroll
    for (int l = 0; l < D; ++l) {
      lo[l] = 1e300;
      hi[l] = -1e300;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      long i = i0 + threadIdx.x + (long)r * BLOCK;
      if (i < iend) {
        const long row = checked_index(xperm ? (long)xperm[checked_index(i, a.nx, a.status)] : i, a.nx, a.status);
#pragma unroll
        for (int l = 0; l < D; ++l) {
          double v = a.x[row * D + l];
          lo[l] = fmin(lo[l], v);
          hi[l] = fmax(hi[l], v);
        }
      }
    }
#pragma unroll
    for (int l = 0; l < D; ++l) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lo[l] = fmin(lo[l], __shfl_xor_sync(0xffffffffu, lo[l], o));
        hi[l] = fmax(hi[l], __shfl_xor_sync(0xffffffffu, hi[l], o));
      }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
      for (int l = 0; l < D; ++l) {
        s_red[l][threadIdx.x >> 5] = lo[l];
        s_red[D + l][threadIdx.x >> 5] = hi[l];
      }
    }
    __syncthreads();
    if (threadIdx.x < D) {
      double mn = 1e300, mx = -1e300;
      for (int w2 = 0; w2 < BLOCK / 32; ++w2) {
        mn = fmin(mn, s_red[threadIdx.x][w2]);
        mx = fmax(mx, s_red[D + threadIdx.x][w2]);
      }
      s_ctr[threadIdx.x] = (CENTER && mn <= mx) ? 0.5 * (mn + mx) : 0.0;
      s_box[threadIdx.x] = mn;
      s_box[D + threadIdx.x] = mx;
    }
    __syncthreads();
#pragma unroll
    for (int l = 0; l < D; ++l) {
      ctr[l] = s_ctr[l];
      ctrf[l] = 0.f;
    }
  } else {
#pragma unroll
    for (int l = 0; l < D; ++l) {
      ctr[l] = 0.0;
      ctrf[l] = 0.f;
    }
  }

  if constexpr (std::is_same<T, f32w>::value) {
    // adaptive two-float coordinates: only a CTA whose targets spread wider than kTwoFloatWidth
    // scaled units pays for the low parts (in the spatial order no tile is that wide)
    double width = 0.0;
    if (packed) {
      width = (double)s_widf;
    } else {
#pragma unroll
      for (int l = 0; l < D; ++l) width = fmax(width, (s_box[D + l] - s_box[l]) * a.xscale);
    }
    if (!(width <= kTwoFloatWidth))
      pair_body<Op, T, D, BLOCK, R, TJ, MERGE, UNR, CSM, true>(a, tile_idx, split, i0, iend, ctr, ctrf, s_box,
                                                                 s_visit, smem_raw);
    else
      pair_body<Op, T, D, BLOCK, R, TJ, MERGE, UNR, CSM, false>(a, tile_idx, split, i0, iend, ctr, ctrf, s_box,
                                                                 s_visit, smem_raw);
  } else {
    pair_body<Op, T, D, BLOCK, R, TJ, MERGE, UNR, CSM, false>(a, tile_idx, split, i0, iend, ctr, ctrf, s_box,
                                                                 s_visit, smem_raw);
  }
}

// Caller order: CTA x takes target tile x. Spatial order: the CTAs loop over the tiles the order
// built (their count is known on the device only; the grid is sized for the usual count).
template <class Op, typename T, int D, int BLOCK, int R, int TJ, int MERGE, int MINB, int UNR, int CSM>
__global__ void __launch_bounds__(BLOCK, MINB) pair_kernel(const PairArgs a) {
  pdl_entry();
  const long nt = a.xtiles ? (long)*a.nxtiles : (long)gridDim.x;
  if constexpr (std::is_same<T, f32b>::value) {
    if ((long)blockIdx.x >= nt) return;  // no tile for this CTA (whole CTA)
    bulk_init();
  }
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    if (t != (long)blockIdx.x) __syncthreads();  // the previous tile is done with shared memory
    pair_block<Op, T, D, BLOCK, R, TJ, MERGE, UNR, CSM>(a, t, (int)blockIdx.y);
    if constexpr (std::is_same<T, f32b>::value) {
      __syncthreads();
      if (!bulk_state().ok) return;  // a bounded wait gave up (reported in a.status)
    }
  }
}

// Batched form: CTA b works on item items[b] = (problem, target tile, source split) of the
// problem's arguments args[problem]. One launch covers every problem of a batch (the subjects of
// an atlas), whatever their sizes; items are ordered by the host (largest first). The host fills
// every field of args, including j_chunk, nsplit, partial and xscale (coord_scale of the lane type).
template <class Op, typename T, int D, int BLOCK, int R, int TJ, int MERGE, int MINB, int UNR, int CSM>
__global__ void __launch_bounds__(BLOCK, MINB) pair_kernel_batched(const PairArgs *args, const int4 *items) {
  pdl_entry();
  const int4 it = items[blockIdx.x];
  const PairArgs a = args[it.x];
  if constexpr (std::is_same<T, f32b>::value) bulk_init();
  pair_block<Op, T, D, BLOCK, R, TJ, MERGE, UNR, CSM>(a, (long)it.y, it.z);
}

// Sums the per-split FP64 partials in split order and applies the op's store.
template <class Op>
__global__ void split_reduce_kernel(const PairArgs a) {
  pdl_entry();
  constexpr int NO = Op::NO;
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nx) return;
  double v[NO];
#pragma unroll
  for (int o = 0; o < NO; ++o) v[o] = 0.0;
  for (int s = 0; s < a.nsplit; ++s) {
    const double *p = a.partial + (long)s * NO * a.nx;
#pragma unroll
    for (int o = 0; o < NO; ++o) v[o] += p[(long)o * a.nx + i];
  }
  Op::store(a, a.xperm ? (long)a.xperm[i] : i, v);
}

// Launch configuration of one pair kernel.
struct LaunchCfg {
  int variant;  // index into the op's compiled (BLOCK, R, TJ) table
  int nsplit;   // source splits (grid.y); 1 = no partial buffer
};

// Batched split reduction: thread over (problem, target) items ritems[b] = (problem, first target).
template <class Op>
__global__ void split_reduce_batched_kernel(const PairArgs *args, const int2 *ritems) {
  pdl_entry();
  constexpr int NO = Op::NO;
  const int2 it = ritems[blockIdx.x];
  const PairArgs &a = args[it.x];
  const long i = (long)it.y + threadIdx.x;
  if (i >= a.nx || a.nsplit <= 1) return;
  double v[NO];
#pragma unroll
  for (int o = 0; o < NO; ++o) v[o] = 0.0;
  for (int s = 0; s < a.nsplit; ++s) {
    const double *p = a.partial + (long)s * NO * a.nx;
#pragma unroll
    for (int o = 0; o < NO; ++o) v[o] += p[(long)o * a.nx + i];
  }
  Op::store(a, a.xperm ? (long)a.xperm[i] : i, v);
}

template <class Op, typename T, int D, int BLOCK, int R, int TJ, int MERGE, int MINB, int UNR, int CSM>
cudaError_t launch_pairs_batched(const PairArgs *args, const int4 *items, int nitems, const int2 *ritems,
                                 int nritems, cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  const size_t smem = pair_smem_bytes<Op, T, D, BLOCK, R, TJ, CSM>();
  auto kern = pair_kernel_batched<Op, T, D, BLOCK, R, TJ, MERGE, MINB, UNR, CSM>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = launch(kern, (unsigned)nitems, BLOCK, smem, st, args, items);
  if (e != cudaSuccess || nritems <= 0) return e;
  return launch(split_reduce_batched_kernel<Op>, (unsigned)nritems, 256, 0, st, args, ritems);
}

template <class Op, typename T, int D, int BLOCK, int R, int TJ, int MERGE, int MINB, int UNR, int CSM>
cudaError_t launch_pairs(PairArgs a, int nsplit, cudaStream_t st) {
  if (a.nx <= 0) return cudaSuccess;
  const size_t smem = pair_smem_bytes<Op, T, D, BLOCK, R, TJ, CSM>();
  auto kern = pair_kernel<Op, T, D, BLOCK, R, TJ, MERGE, MINB, UNR, CSM>;
  a.xscale = coord_scale<T>(a.sigma);
  if (smem > 48 * 1024) {  // per current device; idempotent
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (nsplit < 1) nsplit = 1;
  long per = (a.ny + nsplit - 1) / nsplit;
  per = ((per + TJ - 1) / TJ) * TJ;
  if (per < TJ) per = TJ;
  nsplit = (int)((a.ny + per - 1) / per);
  if (nsplit < 1) nsplit = 1;
  a.j_chunk = per;
  a.nsplit = nsplit;
  if (a.ny == 0) {
    a.j_chunk = TJ;
    a.nsplit = 1;
    nsplit = 1;
  }
  a.prune_d2 = prune_dist2<T>(a.sigma);
  const long tiles = a.xtiles ? a.xtile_bound : (a.nx + (long)BLOCK * R - 1) / ((long)BLOCK * R);
  dim3 grid((unsigned)tiles, (unsigned)nsplit);
  cudaError_t e = launch(kern, grid, BLOCK, smem, st, a);
  if (e != cudaSuccess || nsplit == 1 || a.tickets) return e;
  return launch(split_reduce_kernel<Op>, (unsigned)((a.nx + 255) / 256), 256, 0, st, a);
}

}  // namespace gbk
