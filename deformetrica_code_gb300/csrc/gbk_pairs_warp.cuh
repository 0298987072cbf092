// Warp-split pair kernel for kernel sums too small to fill 152 SMs (control points x control points,
// control points x template vertices): the same operations, lanes, compensation and packed
// coordinates as the small shape of pair_kernel (gbk_pairs.cuh), with a different decomposition.
//
// A CTA owns 32 R targets (R per lane) and one source split (grid.y); its KS warps share those
// targets and divide the split's sources between them, each warp staging its own 32-record tiles
// in its own shared-memory area (synchronised with __syncwarp only: no block barrier in the pair
// loop). At the end the KS warps' compensated sums are added in FP64 in warp order through shared
// memory, then written, or written as the split's partial and reduced by the last split CTA of the
// target tile (the ticket scheme of pair_kernel). Against the small shape (64 threads, 128 targets
// per CTA) this gives a tiny problem KS times more warps per target tile without KS times more
// cross-CTA partials: on 1,000 x 10,242 pairs the small shape keeps ~2 warps per SM busy, and a
// lone warp cannot issue its dependent FP32 chains back to back.
//
// Caller order only (PairArgs::xp / yp must be set: coordinates packed once per launch); no pruning.
// Results are bitwise reproducible run to run (fixed warp and split order).
#pragma once

#include "gbk_dispatch.h"
#include "gbk_pairs.cuh"

namespace gbk {

template <class Op, typename T, int D, int KS, int R, int MERGE, int UNR>
struct WarpShape {
  static constexpr int TJ = 32;  // one staged record per lane
  static constexpr int NJP = Rec<Op, D, T>::NJP;
  static constexpr int TILE = 32 * R;  // targets per CTA
  static constexpr size_t kStage = (size_t)KS * TJ * NJP * sizeof(typename SrcLane<T>::SV);
  static constexpr size_t kReduce = (size_t)KS * Op::NO * TILE * sizeof(double);
  static constexpr size_t kSmem = kStage > kReduce ? kStage : kReduce;  // the reduction reuses the tiles
};

// The pair loop of one warp over sources [jw, jwe) with the CTA's centre c (scaled units).
template <class Op, typename T, int D, int KS, int R, int MERGE, int UNR, bool TWOF>
__device__ __forceinline__ void warp_body(const PairArgs &a, const long i0, const long iend, const long jw,
                                          const long jwe, const float *c, unsigned char *smem) {
  typedef Lane<T> L;
  typedef typename L::V V;
  typedef typename SrcLane<T>::SV SV;
  typedef WarpShape<Op, T, D, KS, R, MERGE, UNR> S;
  constexpr int W = L::kWidth;
  constexpr int G = R / W;
  constexpr int TJ = S::TJ;
  constexpr int LO = D + Op::NS;
  constexpr int NJ = D + Op::NS + (TWOF ? D : 0);
  constexpr int PER16 = 16 / (int)sizeof(SV);
  constexpr int NJP = (NJ + PER16 - 1) / PER16 * PER16;  // the one-float loop reads no low parts
  constexpr int NO = Op::NO;
  static_assert(NJP <= S::NJP, "the warp's tile is sized for the widest record");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  SV *tile = reinterpret_cast<SV *>(smem) + (size_t)warp * TJ * S::NJP;

  V xg[G][D], xlo[G][TWOF ? D : 1], tg[G][Op::NT > 0 ? Op::NT : 1];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    float qh[W][D], ql[W][D];
    double tv[W][Op::NT > 0 ? Op::NT : 1];
#pragma unroll
    for (int w2 = 0; w2 < W; ++w2) {
      const long i = i0 + lane + (long)(g * W + w2) * 32;
      // out-of-range lanes compute a copy, never stored
      const long ic = checked_index(i < iend ? i : (iend - 1), a.nx, a.status);
#pragma unroll
      for (int l = 0; l < D; ++l) centre_packed(a.xp[ic * D + l], c[l], qh[w2][l], ql[w2][l]);
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

  V acc[G][NO], sum[G][NO], cmp[G][NO];
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int o = 0; o < NO; ++o) acc[g][o] = sum[g][o] = cmp[g][o] = L::zero();
  const V cx = exp_arg_scale<T>(a.sigma);
  const int p0 = a.p0, p1 = a.p1;

  for (long jt = jw; jt < jwe; jt += TJ) {
    const int cnt = (int)((jwe - jt) < TJ ? (jwe - jt) : TJ);
    {  // stage: lane r converts record r, -(y' - c) and the extras; empty slots are exact no-ops
      SV rv[NJP];
#pragma unroll
      for (int q = 0; q < NJP; ++q) rv[q] = SrcVal<T>::make(0.f);
      if (lane < cnt) {
        const long j = checked_index(jt + lane, a.ny, a.status);
        double ex[Op::NS > 0 ? Op::NS : 1];
        Op::load_source(a, j, ex);
#pragma unroll
        for (int l = 0; l < D; ++l) {
          float qh, ql;
          centre_packed(a.yp[j * D + l], c[l], qh, ql);
          rv[l] = SrcVal<T>::make(-qh);
          if (TWOF) rv[LO + l < NJP ? LO + l : 0] = SrcVal<T>::make(-ql);
        }
#pragma unroll
        for (int k = 0; k < Op::NS; ++k) rv[D + k] = SrcVal<T>::make(ex[k]);
      }
#pragma unroll
      for (int q = 0; q < NJP; ++q) tile[lane * NJP + q] = rv[q];
    }
    __syncwarp();
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
          if (TWOF) {
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
          Comp<T>::fold(sum[g][o], cmp[g][o], acc[g][o]);
          acc[g][o] = L::zero();
        }
    }
    __syncwarp();  // every lane is done with the tile before it is restaged
  }

  // ---- this warp's FP64 sums into the CTA's reduction area (the staging tiles are reused) ----
  __syncthreads();  // every warp is done with its tiles
  double *red = reinterpret_cast<double *>(smem);
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int w2 = 0; w2 < W; ++w2) {
      const int t = lane + (g * W + w2) * 32;
#pragma unroll
      for (int o = 0; o < NO; ++o)
        red[((size_t)warp * NO + o) * S::TILE + t] = (double)L::get(sum[g][o], w2) + (double)L::get(cmp[g][o], w2);
    }
}

template <class Op, typename T, int D, int KS, int R, int MERGE, int UNR, int MINB>
__global__ void __launch_bounds__(32 * KS, MINB) pair_kernel_warp(const PairArgs a) {
  pdl_entry();
  typedef WarpShape<Op, T, D, KS, R, MERGE, UNR> S;
  constexpr int NO = Op::NO;
  constexpr int TILE = S::TILE;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long i0 = (long)blockIdx.x * TILE;
  const long iend = i0 + TILE < a.nx ? i0 + TILE : a.nx;
  const int split = (int)blockIdx.y;

  // ---- centre: the box of the tile's packed high parts, reduced in every warp alike (no barrier) ----
  float c[D], wid = 0.f;
#pragma unroll
  for (int l = 0; l < D; ++l) {
    float lo = 3.0e38f, hi = -3.0e38f;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const long i = i0 + lane + (long)r * 32;
      if (i < iend) {
        const float v = a.xp[checked_index(i, a.nx, a.status) * D + l].x;
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    c[l] = lo <= hi ? 0.5f * lo + 0.5f * hi : 0.f;
    wid = fmaxf(wid, hi - lo);  // an infinite spread makes the tile wide (NaN is ignored)
  }

  // ---- this warp's share of the split's sources: whole 32-record tiles, warp by warp ----
  const long jb = (long)split * a.j_chunk;
  const long je = jb + a.j_chunk < a.ny ? jb + a.j_chunk : a.ny;
  const long span = je > jb ? je - jb : 0;
  const long per = ((span + KS - 1) / KS + 31) / 32 * 32;
  const long jw = jb + (long)warp * per < je ? jb + (long)warp * per : je;
  const long jwe = jw + per < je ? jw + per : je;
  if constexpr (std::is_same<T, f32w>::value) {
    if (!(wid <= kTwoFloatWidth))
      warp_body<Op, T, D, KS, R, MERGE, UNR, true>(a, i0, iend, jw, jwe, c, smem_raw);
    else
      warp_body<Op, T, D, KS, R, MERGE, UNR, false>(a, i0, iend, jw, jwe, c, smem_raw);
  } else {
    warp_body<Op, T, D, KS, R, MERGE, UNR, false>(a, i0, iend, jw, jwe, c, smem_raw);
  }
  if (a.pair_count && threadIdx.x == 0 && span > 0)
    atomicAdd(a.pair_count, (unsigned long long)(iend - i0) * (unsigned long long)span);
  __syncthreads();  // every warp's sums are in the reduction area

  // ---- the warps' sums in warp order: the split's result (or its partial) per target ----
  const double *red = reinterpret_cast<const double *>(smem_raw);
  for (int t = threadIdx.x; t < TILE; t += 32 * KS) {
    const long i = i0 + t;
    if (i >= iend) continue;
    double v[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) v[o] = red[(size_t)o * TILE + t];
    for (int w = 1; w < KS; ++w) {
#pragma unroll
      for (int o = 0; o < NO; ++o) v[o] += red[((size_t)w * NO + o) * TILE + t];
    }
    if (a.nsplit > 1) {
      double *p = a.partial + (long)split * NO * a.nx;
#pragma unroll
      for (int o = 0; o < NO; ++o) p[(long)o * a.nx + i] = v[o];
    } else {
      Op::store(a, i, v);
    }
  }
  if (a.nsplit > 1) {
    // the last split CTA of the tile sums the partials in split order (see pair_body)
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      s_last = atomicAdd(a.tickets + blockIdx.x, 1u) == (unsigned)(a.nsplit - 1);
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      constexpr int SB = NO >= 24 ? 1 : 24 / NO;
      for (int t = threadIdx.x; t < TILE; t += 32 * KS) {
        const long i = i0 + t;
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
        Op::store(a, i, v);
      }
      if (threadIdx.x == 0) a.tickets[blockIdx.x] = 0u;
    }
  }
}

// Launch: grid (target tiles, nsplit); each split a whole number of KS x 32 sources.
template <class Op, typename T, int D, int KS, int R, int MERGE, int UNR, int MINB>
cudaError_t launch_pairs_warp(PairArgs a, int nsplit, cudaStream_t st) {
  typedef WarpShape<Op, T, D, KS, R, MERGE, UNR> S;
  if (a.nx <= 0) return cudaSuccess;
  if (!a.xp || !a.yp || a.xperm || a.yperm || a.xtiles || (nsplit > 1 && !a.tickets)) return cudaErrorInvalidValue;
  auto kern = pair_kernel_warp<Op, T, D, KS, R, MERGE, UNR, MINB>;
  a.xscale = coord_scale<T>(a.sigma);
  if (S::kSmem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::kSmem);
    if (e != cudaSuccess) return e;
  }
  if (nsplit < 1) nsplit = 1;
  const long unit = (long)KS * S::TJ;
  long per = (a.ny + nsplit - 1) / nsplit;
  per = ((per + unit - 1) / unit) * unit;
  if (per < unit) per = unit;
  nsplit = a.ny > 0 ? (int)((a.ny + per - 1) / per) : 1;
  a.j_chunk = per;
  a.nsplit = nsplit;
  const long tiles = (a.nx + S::TILE - 1) / S::TILE;
  return launch(kern, dim3((unsigned)tiles, (unsigned)nsplit), 32 * KS, S::kSmem, st, a);
}

// Records one compiled warp-split kernel in the host table (see set_entry in gbk_dispatch.h): KS warps
// per CTA, R targets per lane, compensation runs of MERGE sources, UNR-way unrolled source loop, MINB
// resident CTAs per SM requested from the register allocator.
template <class OpT, typename T, int D, int KS, int R, int MERGE, int UNR, int MINB>
inline bool set_entry_warp(KernelEntry *e) {
  typedef WarpShape<OpT, T, D, KS, R, MERGE, UNR> S;
  e->fn = &launch_pairs_warp<OpT, T, D, KS, R, MERGE, UNR, MINB>;
  e->fnb = nullptr;
  e->kernel = (const void *)&pair_kernel_warp<OpT, T, D, KS, R, MERGE, UNR, MINB>;
  e->block = 32 * KS;
  e->r = R;
  e->tj = S::TJ;
  e->no = OpT::NO;
  e->smem = (int)S::kSmem;
  e->packable = true;
  e->tile = S::TILE;
  e->ks = KS;
  return true;
}

}  // namespace gbk
