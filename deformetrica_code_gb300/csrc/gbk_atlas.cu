// Batched deterministic-atlas iteration: every subject's shooting, flow, data term and adjoint in
// one launch per stage, replayed from one CUDA graph.
//
// The reference runs one CPU thread per subject, each making its own kernel calls
// (AbstractAtlas.cxx:138-205 forward, :489-613 gradient, itk::MultiThreader at :782-822). Here the
// subjects of an iteration share every launch: a stage (e.g. "Euler step t of the shooting") is one
// batched pair-kernel launch whose work list holds (subject, target tile, source split) items for
// all subjects, and the FP64 element-wise work between stages is one batched kernel. Subjects may
// have different target meshes (uneven vertex and face counts): the cross data-term pass cuts every
// subject's target faces into source chunks of one common size, so that items cost about the same,
// and the list is ordered largest first. The template (vertices, faces) and the control points are
// shared; each subject has its own momenta.
//
// Per subject s (DeterministicAtlas.cxx:99-154, :246-280; AbstractAtlas.cxx:559-613):
//   L_s = -0.5 match_s / data_sigma2 - 0.5 <K p_s, p_s>,
//   dL/dp_s = -xi_mom_s(0) - K p_s,
// and over the population dL/dcp = sum_s (-xi_pos_s(0) - ConvolveGradient(cp, p_s)) and the
// template vertex gradient sum_s -theta_s(0) (AbstractAtlas.cxx:605-611), summed in subject order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_dispatch.h"
#include "gbk_geometry.h"
#include "gbk_ops.h"
#include "gbk_optimize.h"

using namespace gbk;

namespace {

unsigned nb(long n, int bs = 256) { return (unsigned)std::max(1L, (n + bs - 1) / bs); }

// out[s] = base[s] + c1 v1[s] + c2 v2[s] for s < S, n doubles each, per-array subject strides; a
// subject whose flag is set copies flag_value (or base) instead (nearly zero momenta).
__global__ void lincomb_batched_kernel(int S, long n, double *out, long so, const double *base, long sb,
                                       double c1, const double *v1, long s1, double c2, const double *v2,
                                       long s2, const int *flag, const double *flag_value, long sf) {
  pdl_entry();
  long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long)S * n) return;
  const long s = k / n, i = k % n;
  if (flag && flag[s]) {
    out[s * so + i] = flag_value ? flag_value[s * sf + i] : (base ? base[s * sb + i] : 0.0);
    return;
  }
  double r = base ? base[s * sb + i] : 0.0;
  if (v1) r += c1 * v1[s * s1 + i];
  if (v2) r += c2 * v2[s * s2 + i];
  out[s * so + i] = r;
}

// flag[s] = (|p_s|_F < 1e-20), one CTA per subject
__global__ void __launch_bounds__(256) norm_flag_batched_kernel(const double *p, long n, long stride, int *flag) {
  pdl_entry();
  __shared__ double sh[256];
  const double *q = p + (long)blockIdx.x * stride;
  double acc = 0.0;
  for (long i = threadIdx.x; i < n; i += blockDim.x) acc = fma(q[i], q[i], acc);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) flag[blockIdx.x] = sqrt(sh[0]) < 1e-20 ? 1 : 0;
}

__global__ void zero_flagged_kernel(int S, long n, double *p, long stride, const int *flag) {
  pdl_entry();
  long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long)S * n) return;
  const long s = k / n;
  if (flag[s]) p[s * stride + k % n] = 0.0;
}

// out[s] = sum_i a[s][i] b[s][i] in FP64, one CTA per subject, fixed order
__global__ void __launch_bounds__(256) dot_batched_kernel(const double *a, long sa, const double *b, long sbb,
                                                          long n, double *out, int out_stride) {
  pdl_entry();
  __shared__ double sh[256];
  const double *x = a + (long)blockIdx.x * sa, *y = b + (long)blockIdx.x * sbb;
  double acc = 0.0;
  for (long i = threadIdx.x; i < n; i += blockDim.x) acc = fma(x[i], y[i], acc);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[(long)blockIdx.x * out_stride] = sh[0];
}

// per-subject log-likelihood terms and totals (subject order)
__global__ void loglik_kernel(int S, const double *norm_t, const double *ss, const double *st, const double *kpp,
                              double inv2s2, double *match, double *out) {
  pdl_entry();
  if (threadIdx.x != 0) return;
  double tot = 0.0, data = 0.0, reg = 0.0;
  for (int s = 0; s < S; ++s) {
    const double m = norm_t[s] + ss[s] - 2.0 * st[s];
    match[s] = m;
    const double ld = -m * inv2s2, lr = -0.5 * kpp[s];
    out[3 + s] = ld + lr;
    data += ld;
    reg += lr;
    tot += ld + lr;
  }
  out[0] = tot;
  out[1] = data;
  out[2] = reg;
}

// out[i] = sum_s (c1 a[s][i] + c2 b[s][i]) in subject order
__global__ void sum_subjects_kernel(int S, long n, double *out, const double *a, long sa, double c1, const double *b,
                                    long sbb, double c2) {
  pdl_entry();
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double r = 0.0;
  for (int s = 0; s < S; ++s) {
    if (a) r += c1 * a[s * sa + i];
    if (b) r += c2 * b[s * sbb + i];
  }
  out[i] = r;
}

// template faces of every subject's deformed template: centres, normals (+ varifold tensors)
__global__ void face_batched_kernel(int S, const double *pts, long spts, const int *tris, long nf, int kind,
                                    double *c, double *n, double *mn, double *w) {
  pdl_entry();
  long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long)S * nf) return;
  const long s = k / nf, f = k % nf;
  const double *P = pts + s * spts;
  const int i0 = tris[3 * f], i1 = tris[3 * f + 1], i2 = tris[3 * f + 2];
  double a[3], b[3], nn[3];
  for (int q = 0; q < 3; ++q) {
    a[q] = P[3 * i2 + q] - P[3 * i0 + q];
    b[q] = P[3 * i1 + q] - P[3 * i0 + q];
    c[3 * k + q] = (P[3 * i0 + q] + P[3 * i1 + q] + P[3 * i2 + q]) / 3.0;
  }
  nn[0] = 0.5 * (a[1] * b[2] - a[2] * b[1]);
  nn[1] = 0.5 * (a[2] * b[0] - a[0] * b[2]);
  nn[2] = 0.5 * (a[0] * b[1] - a[1] * b[0]);
  if (kind == 1) {
    const double sc = 1.0 / sqrt(sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]) + 1e-20);
    for (int q = 0; q < 3; ++q) nn[q] *= sc;
    double *m6 = mn + 6 * k, *w6 = w + 6 * k;
    m6[0] = nn[0] * nn[0];
    m6[1] = nn[0] * nn[1];
    m6[2] = nn[0] * nn[2];
    m6[3] = nn[1] * nn[1];
    m6[4] = nn[1] * nn[2];
    m6[5] = nn[2] * nn[2];
    w6[0] = m6[0];
    w6[1] = 2 * m6[1];
    w6[2] = 2 * m6[2];
    w6[3] = m6[3];
    w6[4] = 2 * m6[4];
    w6[5] = m6[5];
  }
  for (int q = 0; q < 3; ++q) n[3 * k + q] = nn[q];
}

__device__ inline void sym6(const double *m, const double *x, double *y) {
  y[0] = m[0] * x[0] + m[1] * x[1] + m[2] * x[2];
  y[1] = m[1] * x[0] + m[3] * x[1] + m[4] * x[2];
  y[2] = m[2] * x[0] + m[4] * x[1] + m[5] * x[2];
}

__global__ void face_grad_batched_kernel(long total, int kind, int dw, const double *n, const double *mn,
                                         const double *kts, const double *ktt, const double *gs, const double *gt,
                                         double *kt, double *gk) {
  pdl_entry();
  long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  if (kind == 0) {
    for (int q = 0; q < 3; ++q) {
      kt[3 * k + q] = kts[3 * k + q] - ktt[3 * k + q];
      gk[3 * k + q] = (gs[3 * k + q] - gt[3 * k + q]) * 2.0 / 3.0;
    }
    return;
  }
  const double *nf = n + 3 * k;
  const double m2 = nf[0] * nf[0] + nf[1] * nf[1] + nf[2] * nf[2];
  if (!(m2 > 1e-20)) {
    for (int q = 0; q < 3; ++q) kt[3 * k + q] = gk[3 * k + q] = 0.0;
    return;
  }
  double dk[6], v[3], aux[3];
  for (int q = 0; q < 6; ++q) dk[q] = kts[6 * k + q] - ktt[6 * k + q];
  sym6(dk, nf, v);
  for (int q = 0; q < 3; ++q) v[q] *= 2.0;
  sym6(mn + 6 * k, v, aux);
  const double inv = 1.0 / sqrt(m2);
  for (int q = 0; q < 3; ++q) {
    kt[3 * k + q] = (v[q] - aux[q] / (2.0 * m2)) * inv;
    gk[3 * k + q] = (gs[3 * k + q] - gt[3 * k + q]) * (2.0 / 3.0);
  }
}

// theta_T[s][v] = scale * sum over (face, corner) of v: e x kt_f + gk_f (CSR order)
__global__ void vertex_gather_batched_kernel(int S, long nv, long nf, const double *pts, long spts, const int *tris,
                                             const int *ptr, const int *fc, const double *kt, const double *gk,
                                             double *out, long sout, double scale) {
  pdl_entry();
  long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long)S * nv) return;
  const long s = k / nv, v = k % nv;
  const double *P = pts + s * spts;
  const double *KT = kt + s * nf * 3, *GK = gk + s * nf * 3;
  double g[3] = {0.0, 0.0, 0.0};
  for (int q = ptr[v]; q < ptr[v + 1]; ++q) {
    const int f = fc[q] / 3, corner = fc[q] % 3;
    const int a = tris[3 * f + (corner + 2) % 3], b = tris[3 * f + (corner + 1) % 3];
    double e[3];
    for (int t = 0; t < 3; ++t) e[t] = P[3 * a + t] - P[3 * b + t];
    const double *t3 = KT + 3 * f;
    g[0] += e[1] * t3[2] - e[2] * t3[1] + GK[3 * f + 0];
    g[1] += e[2] * t3[0] - e[0] * t3[2] + GK[3 * f + 1];
    g[2] += e[0] * t3[1] - e[1] * t3[0] + GK[3 * f + 2];
  }
  for (int t = 0; t < 3; ++t) out[s * sout + 3 * v + t] = scale * g[t];
}

}  // namespace

// One batched pair launch: per-subject arguments, work list and reduction list.
struct BatchLaunch {
  int op = 0, dv = 3;
  KernelEntry e;
  std::vector<PairArgs> args;  // host copies until upload()
  std::vector<int4> items;
  std::vector<int2> ritems;
  PairArgs *d_args = nullptr;
  int4 *d_items = nullptr;
  int2 *d_ritems = nullptr;
  int nitems = 0, nritems = 0;
};

struct gbk_atlas {
  gbk_ctx *c = nullptr;
  int S = 0, T = 2, heun = 1, kind = 0, dw = 3, use_graph = 1, steps = 0;
  long ncp = 0, nv = 0, nf = 0;
  double sigma_def = 1, sigma_data = 1, data_sigma2 = 1;
  double smoothing = 0.0;  // template-gradient smoothing width (0: the L2 gradient)
  int lag = 1;             // the optimiser deforms the reference's lagged template
  std::vector<long> nft;  // target faces per subject
  cudaStream_t stream = nullptr;
  std::vector<void *> owned;
  std::vector<BatchLaunch> launches;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long graph_kernels = 0;
  // device arrays ([S][...] blocks)
  double *cp = nullptr, *mom = nullptr;                         // ncp x 3, S x ncp x 3
  double *pos = nullptr, *momt = nullptr, *xp = nullptr, *xm = nullptr;  // S x T x ncp x 3
  double *lm0 = nullptr, *lm = nullptr, *theta = nullptr;       // nv x 3, S x T x nv x 3
  double *va = nullptr, *vb = nullptr, *vc = nullptr, *vd = nullptr;  // S x max(ncp, nv) x 3
  double *kp = nullptr, *greg = nullptr, *gmom = nullptr, *gcp = nullptr, *gtmpl = nullptr, *gtmpl_l2 = nullptr;
  // the points the template gradient is smoothed over (the current fixed-effect template, = lm0
  // outside the optimiser), and the optimiser's current fixed-effect template (lag)
  double *smooth = nullptr, *tmpl_fe = nullptr;
  double *thT = nullptr;                                        // S x nv x 3
  int *flag = nullptr, *tris = nullptr, *csr_ptr = nullptr, *csr_fc = nullptr;
  double *cs = nullptr, *ns = nullptr, *mns = nullptr, *ws = nullptr;   // S x nf x {3,6}
  double *kts = nullptr, *ktt = nullptr, *gs = nullptr, *gt = nullptr, *kt = nullptr, *gk = nullptr;
  double *ct = nullptr, *tw = nullptr;  // concatenated target faces: centres, weights (n or MN)
  std::vector<long> toff;               // face offset of each subject's target
  double *norm_t = nullptr, *dot_ss = nullptr, *dot_st = nullptr, *kpp = nullptr, *match = nullptr, *out = nullptr;
  double *partial = nullptr;
  size_t partial_per_subject = 0;
  long rows = 0;

  template <class P>
  int alloc(P **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max(count * sizeof(P), (size_t)8));
    if (e != cudaSuccess) return c->cuda(e, "cudaMalloc (atlas)");
    owned.push_back(q);
    *p = (P *)q;
    return GBK_OK;
  }

  // Adds a batched launch (host side). Uniform stages are split for >= 2 waves over all subjects;
  // the uneven stage (chunk > 0) cuts every subject's sources into chunks of `chunk`.
  int add_launch(int op, int dv, std::vector<PairArgs> &args, long chunk) {
    BatchLaunch L;
    L.op = op;
    L.dv = dv;
    // Convolve-like stages run the adaptive two-float variant (FP32C): a CTA whose targets spread
    // wider than 16 scaled units forms its differences from hi + lo coordinates, any other CTA runs
    // the one-float loop; the other stages run the default variant
    if (!find_kernel(op, c->mode, 3, dv, VARIANT_TWO_FLOAT, &L.e) && !find_kernel(op, c->mode, 3, dv, 0, &L.e))
      return c->fail(GBK_ERR_UNSUPPORTED, "atlas: no kernel op %d dv %d", op, dv);
    const long per = (long)L.e.block * L.e.r;
    int occ = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, L.e.kernel, L.e.block, L.e.smem) != cudaSuccess) occ = 1;
    cudaGetLastError();
    const long slots = (long)c->num_sms * std::max(occ, 1);
    struct Item {
      int s, tile, split;
      long cost;
    };
    std::vector<Item> items;
    for (int s = 0; s < S; ++s) {
      PairArgs &a = args[s];
      const long itiles = (a.nx + per - 1) / per;
      long jc;
      if (chunk > 0) {
        jc = ((chunk + L.e.tj - 1) / L.e.tj) * L.e.tj;
      } else {
        const long total_tiles = (long)S * itiles;
        long want = std::max(1L, (2 * slots + total_tiles - 1) / total_tiles);
        want = std::min(want, std::max(1L, a.ny / (2L * L.e.tj)));
        jc = (a.ny + want - 1) / want;
        jc = ((jc + L.e.tj - 1) / L.e.tj) * L.e.tj;
      }
      jc = std::max(jc, (long)L.e.tj);
      const int nsplit = (int)std::max(1L, (a.ny + jc - 1) / jc);
      a.j_chunk = jc;
      a.nsplit = nsplit;
      a.partial = nullptr;  // patched in upload()
      // coordinate pre-scale of the lane type (the single-problem launcher sets it itself)
      a.xscale = c->mode == MODE_F64 ? coord_scale<double>(a.sigma) : coord_scale<float>(a.sigma);
      a.pair_count = c->pair_counter_of(op);  // evaluated pairs, by operation (gbk_evaluated_pairs_by_op)
      if (nsplit > 1) partial_per_subject = std::max(partial_per_subject, (size_t)nsplit * L.e.no * a.nx);
      for (long t = 0; t < itiles; ++t)
        for (int sp = 0; sp < nsplit; ++sp) items.push_back({s, (int)t, sp, std::min(jc, a.ny - (long)sp * jc)});
      if (nsplit > 1)
        for (long i0 = 0; i0 < a.nx; i0 += 256) L.ritems.push_back(make_int2(s, (int)i0));
    }
    std::stable_sort(items.begin(), items.end(), [](const Item &x, const Item &y) { return x.cost > y.cost; });
    for (const Item &it : items) L.items.push_back(make_int4(it.s, it.tile, it.split, 0));
    L.args = args;
    L.nitems = (int)L.items.size();
    L.nritems = (int)L.ritems.size();
    launches.push_back(std::move(L));
    return GBK_OK;
  }

  // Allocates the per-subject partial buffers at the size the split plan needs and uploads the
  // argument tables and work lists.
  int upload() {
    int rc = alloc(&partial, (size_t)S * std::max(partial_per_subject, (size_t)1));
    for (BatchLaunch &L : launches) {
      if (rc) break;
      for (int s = 0; s < S; ++s)
        if (L.args[s].nsplit > 1) L.args[s].partial = partial + (size_t)s * partial_per_subject;
      if ((rc = alloc(&L.d_args, L.args.size()))) break;
      if ((rc = alloc(&L.d_items, L.items.size()))) break;
      if ((rc = alloc(&L.d_ritems, std::max<size_t>(L.ritems.size(), 1)))) break;
      rc = c->cuda(cudaMemcpy(L.d_args, L.args.data(), L.args.size() * sizeof(PairArgs), cudaMemcpyHostToDevice), "H2D");
      if (!rc) rc = c->cuda(cudaMemcpy(L.d_items, L.items.data(), L.items.size() * sizeof(int4), cudaMemcpyHostToDevice), "H2D");
      if (!rc && !L.ritems.empty())
        rc = c->cuda(cudaMemcpy(L.d_ritems, L.ritems.data(), L.ritems.size() * sizeof(int2), cudaMemcpyHostToDevice), "H2D");
      L.args.clear();
      L.items.clear();
      L.ritems.clear();
    }
    return rc;
  }

  int run_launch(size_t k) {
    const BatchLaunch &L = launches[k];
    int rc = c->cuda(L.e.fnb(L.d_args, L.d_items, L.nitems, L.d_ritems, L.nritems, stream), "batched pair launch");
    c->launches += L.nritems ? 2 : 1;
    return rc;
  }

  // launch order is fixed at build time; body() replays it with the element-wise kernels between
  int body();
  int build_launches();
  // one iteration on `stream`: eager at first, captured the second time, replayed afterwards
  int run() {
    cudaStream_t saved = c->stream;
    c->stream = stream;
    gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
    int rc = GBK_OK;
    if (!use_graph || steps == 0) {
      rc = body();
    } else {
      if (!exec) {
        long long l0 = c->launches;
        rc = c->cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        if (!rc) {
          rc = body();
          cudaGraph_t g = nullptr;
          cudaError_t e = cudaStreamEndCapture(stream, &g);
          if (!rc && e != cudaSuccess) rc = c->cuda(e, "end capture");
          if (!rc) rc = c->cuda(cudaGraphInstantiate(&exec, g, 0), "graph instantiate");
          graph = g;
          graph_kernels = c->launches - l0;
          c->launches = l0;
        }
      }
      if (!rc) {
        rc = c->cuda(cudaGraphLaunch(exec, stream), "graph launch");
        c->launches += graph_kernels;
      }
    }
    c->stream = saved;
    if (!rc) ++steps;
    return rc;
  }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    steps = 0;
  }
  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    for (void *p : owned) cudaFree(p);
    owned.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

static PairArgs pa(long nx, long ny, double sigma) { return pair_args(nx, ny, sigma); }

// Builds, in execution order, the batched launches of one iteration.
int gbk_atlas::build_launches() {
  const long n = ncp * 3, m = nv * 3, sT_n = (long)T * n, sT_m = (long)T * m;
  std::vector<PairArgs> A(S);
  int rc;
  // shooting: step t, fused Convolve + alpha-gradient CP x CP; step 0 writes K p, G^T p for the
  // regularity term as well
  for (int t = 0; t + 1 < T; ++t) {
    for (int s = 0; s < S; ++s) {
      PairArgs a = pa(ncp, ncp, sigma_def);
      a.x = pos + s * sT_n + t * n;
      a.y = a.x;
      a.w = momt + s * sT_n + t * n;
      a.w_ld = 3;
      a.ta = a.w;
      a.ta_ld = 3;
      a.out0 = (t == 0 ? kp : va) + s * rows * 3;
      a.out0_ld = 3;
      a.out1 = (t == 0 ? greg : vb) + s * rows * 3;
      a.out1_ld = 3;
      A[s] = a;
    }
    if ((rc = add_launch(OP_CONV_GRADA, 3, A, 0))) return rc;
  }
  // flow: Convolve V x CP at t (and t + 1 for Heun)
  for (int t = 0; t + 1 < T; ++t)
    for (int stage = 0; stage < (heun ? 2 : 1); ++stage) {
      for (int s = 0; s < S; ++s) {
        PairArgs a = pa(nv, ncp, sigma_def);
        a.x = lm + s * sT_m + (t + stage) * m;
        a.y = pos + s * sT_n + (t + stage) * n;
        a.w = momt + s * sT_n + (t + stage) * n;
        a.w_ld = 3;
        a.out0 = (stage == 0 ? vc : vd) + s * rows * 3;
        a.out0_ld = 3;
        A[s] = a;
      }
      if ((rc = add_launch(OP_CONV, 3, A, 0))) return rc;
    }
  // data term: self pass (uniform) and cross pass (uneven target sizes, chunked sources)
  const double *alpha = kind ? ws : ns, *wsrc = kind ? mns : ns;
  for (int s = 0; s < S; ++s) {
    PairArgs a = pa(nf, nf, sigma_data);
    a.x = cs + s * nf * 3;
    a.ta = alpha + s * nf * dw;
    a.ta_ld = dw;
    a.y = a.x;
    a.w = wsrc + s * nf * dw;
    a.w_ld = dw;
    a.out0 = kts + s * nf * dw;
    a.out0_ld = dw;
    a.out1 = gs + s * nf * 3;
    a.out1_ld = 3;
    A[s] = a;
  }
  if ((rc = add_launch(OP_CONV_GRADA, dw, A, 0))) return rc;
  long tot = 0;
  for (int s = 0; s < S; ++s) tot += nft[s];
  const long tiles = (nf + 511) / 512;
  const long chunk = std::max(512L, tot * tiles / (3L * c->num_sms * 3));
  for (int s = 0; s < S; ++s) {
    PairArgs a = pa(nf, nft[s], sigma_data);
    a.x = cs + s * nf * 3;
    a.ta = alpha + s * nf * dw;
    a.ta_ld = dw;
    a.y = ct + toff[s] * 3;
    a.w = tw + toff[s] * dw;
    a.w_ld = dw;
    a.out0 = ktt + s * nf * dw;
    a.out0_ld = dw;
    a.out1 = gt + s * nf * 3;
    a.out1_ld = 3;
    A[s] = a;
  }
  if ((rc = add_launch(OP_CONV_GRADA, dw, A, chunk))) return rc;
  // landmark adjoint: alpha-gradient V x CP at t (and t - 1 for Heun)
  for (int t = T - 1; t > 0; --t)
    for (int stage = 0; stage < (heun ? 2 : 1); ++stage) {
      const int tt = t - stage;
      for (int s = 0; s < S; ++s) {
        PairArgs a = pa(nv, ncp, sigma_def);
        a.x = lm + s * sT_m + tt * m;
        a.ta = theta + s * sT_m + tt * m;
        a.ta_ld = 3;
        a.y = pos + s * sT_n + tt * n;
        a.w = momt + s * sT_n + tt * n;
        a.w_ld = 3;
        a.out1 = (stage == 0 ? vc : vd) + s * rows * 3;
        a.out1_ld = 3;
        A[s] = a;
      }
      if ((rc = add_launch(OP_GRADA, 3, A, 0))) return rc;
    }
  // diffeo adjoint: ComputeUpdateAt(t) and, with Heun, ComputeUpdateAt(t - 1)
  for (int t = T - 1; t > 0; --t)
    for (int stage = 0; stage < (heun ? 2 : 1); ++stage) {
      const int tt = t - stage;
      double *dpos = stage == 0 ? va : vc, *dmom = stage == 0 ? vb : vd;
      for (int s = 0; s < S; ++s) {
        PairArgs a = pa(ncp, ncp, sigma_def);
        a.x = pos + s * sT_n + tt * n;
        a.y = a.x;
        a.ta = momt + s * sT_n + tt * n;
        a.ta_ld = 3;
        a.w = a.ta;
        a.w_ld = 3;
        a.tb = xp + s * sT_n + tt * n;
        a.tb_ld = 3;
        a.sb = xm + s * sT_n + tt * n;
        a.sb_ld = 3;
        a.out0 = dpos + s * rows * 3;
        a.out0_ld = 3;
        a.out1 = dmom + s * rows * 3;
        a.out1_ld = 3;
        A[s] = a;
      }
      if ((rc = add_launch(OP_ADJCP, 3, A, 0))) return rc;
      for (int s = 0; s < S; ++s) {
        PairArgs b = pa(ncp, nv, sigma_def);
        b.x = pos + s * sT_n + tt * n;
        b.ta = momt + s * sT_n + tt * n;
        b.ta_ld = 3;
        b.y = lm + s * sT_m + tt * m;
        b.w = theta + s * sT_m + tt * m;
        b.w_ld = 3;
        b.out0 = dmom + s * rows * 3;
        b.out0_ld = 3;
        b.acc0 = 1;
        b.out1 = dpos + s * rows * 3;
        b.out1_ld = 3;
        b.acc1 = 1;
        A[s] = b;
      }
      if ((rc = add_launch(OP_CONV_GRADA, 3, A, 0))) return rc;
    }
  return GBK_OK;
}

int gbk_atlas::body() {
  const long n = ncp * 3, m = nv * 3, sT_n = (long)T * n, sT_m = (long)T * m, sr = rows * 3;
  const double dt = 1.0 / (T - 1);
  cudaStream_t st = stream;
  size_t L = 0;
  int rc;
  auto ok = [&](cudaError_t e, const char *what) { return c->cuda(e, what); };
  // trajectories start at the shared control points / template and each subject's momenta
  // (launch errors of the element-wise kernels are read back with cudaGetLastError after each stage)
  (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, pos, sT_n, cp, 0, 0, nullptr, 0, 0,
                    nullptr, 0, nullptr, nullptr, 0);
  (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, momt, sT_n, mom, n, 0, nullptr, 0, 0,
                    nullptr, 0, nullptr, nullptr, 0);
  (void)gbk::launch(lincomb_batched_kernel, nb((long)S * m), 256, 0, st, S, m, lm, sT_m, lm0, 0, 0, nullptr, 0, 0,
                    nullptr, 0, nullptr, nullptr, 0);
  (void)gbk::launch(norm_flag_batched_kernel, S, 256, 0, st, mom, n, n, flag);
  c->launches += 4;
  if ((rc = ok(cudaGetLastError(), "init"))) return rc;
  // shooting (Diffeos.cxx:589-660)
  for (int t = 0; t + 1 < T; ++t) {
    if ((rc = run_launch(L++))) return rc;
    const double *dpos = t == 0 ? kp : va, *dmom = t == 0 ? greg : vb;
    (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, pos + (t + 1) * n, sT_n, pos + t * n,
                      sT_n, dt, dpos, sr, 0, nullptr, 0, flag, cp, 0);
    (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, momt + (t + 1) * n, sT_n, momt + t * n,
                      sT_n, -dt, dmom, sr, 0, nullptr, 0, flag, nullptr, 0);
    c->launches += 2;
  }
  (void)gbk::launch(zero_flagged_kernel, nb((long)S * (T - 1) * n), 256, 0, st, S, (T - 1) * n, momt + n, sT_n, flag);
  c->launches += 1;
  // flow (Diffeos.cxx:661-712)
  for (int t = 0; t + 1 < T; ++t) {
    if ((rc = run_launch(L++))) return rc;
    (void)gbk::launch(lincomb_batched_kernel, nb((long)S * m), 256, 0, st, S, m, lm + (t + 1) * m, sT_m, lm + t * m,
                      sT_m, dt, vc, sr, 0, nullptr, 0, flag, nullptr, 0);
    c->launches += 1;
    if (heun) {
      if ((rc = run_launch(L++))) return rc;
      (void)gbk::launch(lincomb_batched_kernel, nb((long)S * m), 256, 0, st, S, m, lm + (t + 1) * m, sT_m, lm + t * m,
                        sT_m, 0.5 * dt, vc, sr, 0.5 * dt, vd, sr, flag, nullptr, 0);
      c->launches += 1;
    }
  }
  // data term on the deformed templates
  const double *lmT = lm + (T - 1) * m;
  (void)gbk::launch(face_batched_kernel, nb((long)S * nf), 256, 0, st, S, lmT, sT_m, tris, nf, kind, cs, ns, mns, ws);
  c->launches += 1;
  if ((rc = run_launch(L++))) return rc;  // self
  if ((rc = run_launch(L++))) return rc;  // cross
  const double *alpha = kind ? ws : ns;
  (void)gbk::launch(dot_batched_kernel, S, 256, 0, st, alpha, nf * dw, kts, nf * dw, nf * dw, dot_ss, 1);
  (void)gbk::launch(dot_batched_kernel, S, 256, 0, st, alpha, nf * dw, ktt, nf * dw, nf * dw, dot_st, 1);
  (void)gbk::launch(dot_batched_kernel, S, 256, 0, st, kp, sr, mom, n, n, kpp, 1);
  (void)gbk::launch(loglik_kernel, 1, 32, 0, st, S, norm_t, dot_ss, dot_st, kpp, 0.5 / data_sigma2, match, out);
  (void)gbk::launch(face_grad_batched_kernel, nb((long)S * nf), 256, 0, st, (long)S * nf, kind, dw, ns, mns, kts, ktt,
                    gs, gt, kt, gk);
  (void)gbk::launch(vertex_gather_batched_kernel, nb((long)S * nv), 256, 0, st, S, nv, nf, lmT, sT_m, tris, csr_ptr,
                    csr_fc, kt, gk, theta + (T - 1) * m, sT_m, 0.5 / data_sigma2);
  c->launches += 6;
  if ((rc = ok(cudaGetLastError(), "data term"))) return rc;
  // landmark adjoint (AdjointEquationsIntegrator.cxx:59-136)
  for (int t = T - 1; t > 0; --t) {
    if ((rc = run_launch(L++))) return rc;
    (void)gbk::launch(lincomb_batched_kernel, nb((long)S * m), 256, 0, st, S, m, theta + (t - 1) * m, sT_m,
                      theta + t * m, sT_m, dt, vc, sr, 0, nullptr, 0, nullptr, nullptr, 0);
    c->launches += 1;
    if (heun) {
      if ((rc = run_launch(L++))) return rc;
      (void)gbk::launch(lincomb_batched_kernel, nb((long)S * m), 256, 0, st, S, m, theta + (t - 1) * m, sT_m,
                        theta + t * m, sT_m, 0.5 * dt, vc, sr, 0.5 * dt, vd, sr, nullptr, nullptr, 0);
      c->launches += 1;
    }
  }
  // diffeomorphism-parameter adjoint (:414-570)
  if ((rc = ok(cudaMemsetAsync(xp, 0, (size_t)S * sT_n * sizeof(double), st), "memset"))) return rc;
  if ((rc = ok(cudaMemsetAsync(xm, 0, (size_t)S * sT_n * sizeof(double), st), "memset"))) return rc;
  for (int t = T - 1; t > 0; --t) {
    if ((rc = run_launch(L++))) return rc;
    if ((rc = run_launch(L++))) return rc;
    (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, xp + (t - 1) * n, sT_n, xp + t * n,
                      sT_n, dt, va, sr, 0, nullptr, 0, nullptr, nullptr, 0);
    (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, xm + (t - 1) * n, sT_n, xm + t * n,
                      sT_n, dt, vb, sr, 0, nullptr, 0, nullptr, nullptr, 0);
    c->launches += 2;
    if (heun) {
      if ((rc = run_launch(L++))) return rc;
      if ((rc = run_launch(L++))) return rc;
      (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, xp + (t - 1) * n, sT_n, xp + t * n,
                        sT_n, 0.5 * dt, va, sr, 0.5 * dt, vc, sr, nullptr, nullptr, 0);
      (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, xm + (t - 1) * n, sT_n, xm + t * n,
                        sT_n, 0.5 * dt, vb, sr, 0.5 * dt, vd, sr, nullptr, nullptr, 0);
      c->launches += 2;
    }
  }
  // gradients: dL/dp_s = -xi_mom_s(0) - K p_s ; dL/dcp = sum_s (-xi_pos_s(0) - G_s) ;
  // template: sum_s -theta_s(0)
  (void)gbk::launch(lincomb_batched_kernel, nb((long)S * n), 256, 0, st, S, n, gmom, n, nullptr, 0, -1.0, xm, sT_n,
                    -1.0, kp, sr, nullptr, nullptr, 0);
  (void)gbk::launch(sum_subjects_kernel, nb(n), 256, 0, st, S, n, gcp, xp, sT_n, -1.0, greg, sr, -1.0);
  (void)gbk::launch(sum_subjects_kernel, nb(m), 256, 0, st, S, m, smoothing > 0 ? gtmpl_l2 : gtmpl, theta, sT_m, -1.0,
                    nullptr, 0, 0.0);
  c->launches += 3;
  if (L != launches.size()) return c->fail(GBK_ERR_STATE, "atlas: launch order mismatch");
  if ((rc = ok(cudaGetLastError(), "atlas gradients"))) return rc;
  if (smoothing > 0) {  // Sobolev template gradient: K_smooth(template, template) L2 (ConvolveGradTemplate)
    PairArgs q = pa(nv, nv, smoothing);
    q.x = smooth;
    q.y = smooth;
    q.w = gtmpl_l2;
    q.w_ld = 3;
    q.out0 = gtmpl;
    q.out0_ld = 3;
    if ((rc = c->launch(OP_CONV, 3, 3, q))) return rc;
  }
  return GBK_OK;
}

extern "C" {

int gbk_atlas_create(gbk_ctx *c, long ncp, const double *cp, long nv, const double *tmpl_pts, long nf,
                     const int *tmpl_tris, int nsub, const long *nv_t, const double *tgt_pts,
                     const long *nf_t, const int *tgt_tris, int T, double sigma_def, double sigma_data,
                     double data_sigma2, int data_kind, int heun, gbk_atlas **out) {
  if (!c || !out) return GBK_ERR_ARG;
  *out = nullptr;
  c->err.clear();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (ncp <= 0 || nv <= 0 || nf <= 0 || nsub <= 0 || T < 2) return c->fail(GBK_ERR_ARG, "bad sizes");
  if (!cp || !tmpl_pts || !tmpl_tris || !nv_t || !tgt_pts || !nf_t || !tgt_tris) return c->fail(GBK_ERR_ARG, "null pointer");
  if (data_kind != 0 && data_kind != 1) return c->fail(GBK_ERR_ARG, "data_kind must be 0 (currents) or 1 (varifold)");
  if (!(data_sigma2 > 0)) return c->fail(GBK_ERR_ARG, "data_sigma2 must be positive");
  gbk_atlas *a = new gbk_atlas();
  a->c = c;
  a->S = nsub;
  a->T = T;
  a->heun = heun ? 1 : 0;
  a->kind = data_kind;
  a->dw = data_kind ? 6 : 3;
  a->ncp = ncp;
  a->nv = nv;
  a->nf = nf;
  a->sigma_def = sigma_def;
  a->sigma_data = sigma_data;
  a->data_sigma2 = data_sigma2;
  a->rows = std::max(ncp, nv);
  int rc = c->cuda(cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking), "stream");
  // host copies of the meshes (for CSR lists, offsets and target faces)
  std::vector<int> th((size_t)nf * 3);
  long tot_v = 0, tot_f = 0;
  for (int s = 0; s < nsub; ++s) {
    tot_v += nv_t[s];
    tot_f += nf_t[s];
  }
  std::vector<double> tp((size_t)tot_v * 3);
  std::vector<int> tt((size_t)tot_f * 3);
  if (!rc) {
    cudaMemcpy(th.data(), tmpl_tris, th.size() * sizeof(int), cudaMemcpyDefault);
    cudaMemcpy(tp.data(), tgt_pts, tp.size() * sizeof(double), cudaMemcpyDefault);
    cudaMemcpy(tt.data(), tgt_tris, tt.size() * sizeof(int), cudaMemcpyDefault);
    rc = c->cuda(cudaGetLastError(), "copy meshes");
  }
  for (long q = 0; !rc && q < 3 * nf; ++q)
    if (th[q] < 0 || th[q] >= nv) rc = c->fail(GBK_ERR_ARG, "template triangle index out of range");
  // per subject: target faces (centres, weights) computed on the host in FP64 (once)
  std::vector<double> ct((size_t)tot_f * 3), tw((size_t)tot_f * a->dw);
  a->nft.assign(nf_t, nf_t + nsub);
  a->toff.assign(nsub, 0);
  long voff = 0, foff = 0;
  for (int s = 0; !rc && s < nsub; ++s) {
    a->toff[s] = foff;
    for (long f = 0; f < nf_t[s]; ++f) {
      const int *tr = &tt[(size_t)(foff + f) * 3];
      if (tr[0] < 0 || tr[1] < 0 || tr[2] < 0 || tr[0] >= nv_t[s] || tr[1] >= nv_t[s] || tr[2] >= nv_t[s]) {
        rc = c->fail(GBK_ERR_ARG, "target triangle index out of range (subject %d)", s);
        break;
      }
      const double *p0 = &tp[(size_t)(voff + tr[0]) * 3], *p1 = &tp[(size_t)(voff + tr[1]) * 3],
                   *p2 = &tp[(size_t)(voff + tr[2]) * 3];
      double aa[3], bb[3], nn[3];
      for (int q = 0; q < 3; ++q) {
        aa[q] = p2[q] - p0[q];
        bb[q] = p1[q] - p0[q];
        ct[(size_t)(foff + f) * 3 + q] = (p0[q] + p1[q] + p2[q]) / 3.0;
      }
      nn[0] = 0.5 * (aa[1] * bb[2] - aa[2] * bb[1]);
      nn[1] = 0.5 * (aa[2] * bb[0] - aa[0] * bb[2]);
      nn[2] = 0.5 * (aa[0] * bb[1] - aa[1] * bb[0]);
      double *w = &tw[(size_t)(foff + f) * a->dw];
      if (data_kind == 0) {
        for (int q = 0; q < 3; ++q) w[q] = nn[q];
      } else {
        const double sc = 1.0 / std::sqrt(std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]) + 1e-20);
        for (int q = 0; q < 3; ++q) nn[q] *= sc;
        w[0] = nn[0] * nn[0];
        w[1] = nn[0] * nn[1];
        w[2] = nn[0] * nn[2];
        w[3] = nn[1] * nn[1];
        w[4] = nn[1] * nn[2];
        w[5] = nn[2] * nn[2];
      }
    }
    voff += nv_t[s];
    foff += nf_t[s];
  }
  std::vector<int> ptr, fc;
  if (!rc) build_csr(nv, nf, 3, th.data(), ptr, fc);
  const long n = ncp * 3, m = nv * 3, rows3 = a->rows * 3;
  const size_t S = nsub, TT = T;
  struct {
    double **p;
    size_t count;
  } bufs[] = {{&a->cp, (size_t)n}, {&a->mom, S * n}, {&a->pos, S * TT * n}, {&a->momt, S * TT * n},
              {&a->xp, S * TT * n}, {&a->xm, S * TT * n}, {&a->lm0, (size_t)m}, {&a->lm, S * TT * m},
              {&a->theta, S * TT * m}, {&a->va, S * rows3}, {&a->vb, S * rows3}, {&a->vc, S * rows3},
              {&a->vd, S * rows3}, {&a->kp, S * rows3}, {&a->greg, S * rows3}, {&a->gmom, S * n},
              {&a->gcp, (size_t)n}, {&a->gtmpl, (size_t)m}, {&a->gtmpl_l2, (size_t)m},
              {&a->smooth, (size_t)m}, {&a->tmpl_fe, (size_t)m},
              {&a->cs, S * nf * 3}, {&a->ns, S * nf * 3},
              {&a->mns, S * nf * 6}, {&a->ws, S * nf * 6}, {&a->kts, S * nf * 6}, {&a->ktt, S * nf * 6},
              {&a->gs, S * nf * 3}, {&a->gt, S * nf * 3}, {&a->kt, S * nf * 3}, {&a->gk, S * nf * 3},
              {&a->ct, (size_t)tot_f * 3}, {&a->tw, (size_t)tot_f * a->dw}, {&a->norm_t, S}, {&a->dot_ss, S},
              {&a->dot_st, S}, {&a->kpp, S}, {&a->match, S}, {&a->out, S + 3}};
  for (auto &b : bufs)
    if (!rc) rc = a->alloc(b.p, b.count);
  if (!rc) rc = a->alloc(&a->flag, S);
  if (!rc) rc = a->alloc(&a->tris, (size_t)nf * 3);
  if (!rc) rc = a->alloc(&a->csr_ptr, ptr.size());
  if (!rc) rc = a->alloc(&a->csr_fc, fc.size());
  cudaStream_t saved = c->stream;
  c->stream = a->stream;
  if (!rc) {
    cudaStream_t st = a->stream;
    rc = c->cuda(cudaMemcpyAsync(a->cp, cp, n * sizeof(double), cudaMemcpyDefault, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(a->lm0, tmpl_pts, m * sizeof(double), cudaMemcpyDefault, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(a->smooth, tmpl_pts, m * sizeof(double), cudaMemcpyDefault, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(a->tris, th.data(), th.size() * sizeof(int), cudaMemcpyHostToDevice, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(a->csr_ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(a->csr_fc, fc.data(), fc.size() * sizeof(int), cudaMemcpyHostToDevice, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(a->ct, ct.data(), ct.size() * sizeof(double), cudaMemcpyHostToDevice, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(a->tw, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice, st), "copy");
    if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  }
  // |T_s|^2 once per subject: one Convolve of the target faces, FP64 dot. Temporaries sized by the
  // largest target, released after creation.
  long max_ft = 0;
  for (int s = 0; s < nsub; ++s) max_ft = std::max(max_ft, nf_t[s]);
  double *kw = nullptr, *wdev = nullptr;
  if (!rc) rc = c->cuda(cudaMalloc(&kw, (size_t)max_ft * a->dw * sizeof(double)), "cudaMalloc (target norms)");
  if (!rc) rc = c->cuda(cudaMalloc(&wdev, (size_t)max_ft * 6 * sizeof(double)), "cudaMalloc (target norms)");
  std::vector<double> wd;
  for (int s = 0; !rc && s < nsub; ++s) {
    const double *ws_t = a->tw + a->toff[s] * a->dw;
    const long fs = nf_t[s];
    PairArgs q = pair_args(fs, fs, sigma_data);
    q.x = a->ct + a->toff[s] * 3;
    q.y = q.x;
    q.w = ws_t;
    q.w_ld = a->dw;
    q.out0 = kw;
    q.out0_ld = a->dw;
    rc = c->launch(OP_CONV, 3, a->dw, q);
    if (rc) break;
    if (data_kind == 0) {
      rc = c->cuda(dot_f64(a->stream, ws_t, kw, fs * 3, a->norm_t + s, 0), "dot");
    } else {
      // |T|^2 = sum_f w(n~_f) . (K MN)_f, w = MN with the off-diagonal entries doubled
      wd.resize((size_t)fs * 6);
      for (long f = 0; f < fs; ++f)
        for (int q6 = 0; q6 < 6; ++q6) {
          const double v = tw[(size_t)(a->toff[s] + f) * 6 + q6];
          wd[(size_t)f * 6 + q6] = (q6 == 1 || q6 == 2 || q6 == 4) ? 2.0 * v : v;
        }
      rc = c->cuda(cudaMemcpyAsync(wdev, wd.data(), wd.size() * sizeof(double), cudaMemcpyHostToDevice, a->stream), "copy");
      if (!rc) rc = c->cuda(dot_f64(a->stream, wdev, kw, fs * 6, a->norm_t + s, 0), "dot");
    }
    if (!rc) rc = c->cuda(cudaStreamSynchronize(a->stream), "sync");
  }
  if (kw) cudaFree(kw);
  if (wdev) cudaFree(wdev);
  if (!rc) rc = c->cuda(cudaStreamSynchronize(a->stream), "sync");
  if (!rc) rc = a->build_launches();
  if (!rc) rc = a->upload();
  c->stream = saved;
  if (rc) {
    a->release();
    delete a;
    return rc;
  }
  *out = a;
  return GBK_OK;
}

int gbk_atlas_set_graph(gbk_atlas *a, int enable) {
  if (!a) return GBK_ERR_ARG;
  a->use_graph = enable ? 1 : 0;
  return GBK_OK;
}

int gbk_atlas_step(gbk_atlas *a, const double *mom, double *loglik, double *grad_mom, double *grad_cp,
                   double *grad_tmpl) {
  if (!a) return GBK_ERR_ARG;
  gbk_ctx *c = a->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!mom) return c->fail(GBK_ERR_ARG, "null momenta");
  const size_t nb_mom = (size_t)a->S * a->ncp * 3 * sizeof(double);
  int rc = c->cuda(cudaMemcpyAsync(a->mom, mom, nb_mom, cudaMemcpyDefault, a->stream), "copy momenta");
  if (!rc) rc = a->run();
  const size_t n = (size_t)a->ncp * 3 * sizeof(double);
  if (!rc && loglik) rc = c->cuda(cudaMemcpyAsync(loglik, a->out, (a->S + 3) * sizeof(double), cudaMemcpyDefault, a->stream), "copy");
  if (!rc && grad_mom) rc = c->cuda(cudaMemcpyAsync(grad_mom, a->gmom, a->S * n, cudaMemcpyDefault, a->stream), "copy");
  if (!rc && grad_cp) rc = c->cuda(cudaMemcpyAsync(grad_cp, a->gcp, n, cudaMemcpyDefault, a->stream), "copy");
  if (!rc && grad_tmpl)
    rc = c->cuda(cudaMemcpyAsync(grad_tmpl, a->gtmpl, (size_t)a->nv * 3 * sizeof(double), cudaMemcpyDefault, a->stream), "copy");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(a->stream), "sync");
  return rc;
}

long long gbk_atlas_graph_launches(const gbk_atlas *a) { return a ? a->graph_kernels : 0; }

int gbk_atlas_set_lagged_template(gbk_atlas *a, int enable) {
  if (!a) return GBK_ERR_ARG;
  a->lag = enable ? 1 : 0;
  return GBK_OK;
}

int gbk_atlas_set_template_smoothing(gbk_atlas *a, double width) {
  if (!a) return GBK_ERR_ARG;
  if (!(width >= 0)) return a->c->fail(GBK_ERR_ARG, "smoothing width must be >= 0");
  a->smoothing = width < 1e-20 ? 0.0 : width;  // AbstractAtlas.cxx:729: below 1e-20, no smoothing
  a->drop_graph();                            // the iteration changes: capture it again
  return GBK_OK;
}

// FastGradientAscent (gbk_optimize.cu) of the atlas log-likelihood over the groups, in the
// reference's order, ControlPoints, TemplateData (each when optimised) and Momenta (all subjects);
// the template step uses the smoothed template gradient and its squared norm is <L2, smoothed>
// (DeterministicAtlas.cxx:212-234).
int gbk_atlas_optimize(gbk_atlas *a, double *cp, double *tmpl, double *mom, int optimize_cp, int optimize_template,
                       int max_iterations, double initial_step, int max_line_search, double shrink, double expand,
                       double tolerance, int nb_iter_freeze, double *history, int *iterations, double *info) {
  if (!a) return GBK_ERR_ARG;
  gbk_ctx *c = a->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !tmpl || !mom || !history || !iterations) return c->fail(GBK_ERR_ARG, "null pointer");
  const long n = a->ncp * 3, m = a->nv * 3, nm = (long)a->S * n;
  cudaStream_t st = a->stream;
  double *sq_dev = nullptr;
  int rc = c->cuda(cudaMalloc(&sq_dev, 4 * sizeof(double)), "cudaMalloc (optimiser)");
  if (!rc && !optimize_cp) rc = c->cuda(cudaMemcpyAsync(a->cp, cp, n * sizeof(double), cudaMemcpyDefault, st), "copy");
  // the deformed template (lm0), the smoothing points and the current fixed-effect template all
  // start at the initial template
  if (!rc) rc = c->cuda(cudaMemcpyAsync(a->lm0, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(a->smooth, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(a->tmpl_fe, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  const bool lag = a->lag && optimize_template;
  int ng = 0, gcp = -1, gt = -1;
  long sizes[3];
  double *params[3];
  if (optimize_cp) {
    gcp = ng;
    sizes[ng] = n;
    params[ng++] = cp;
  }
  if (optimize_template) {
    gt = ng;
    sizes[ng] = m;
    params[ng++] = tmpl;
  }
  const int gm = ng;
  sizes[ng] = nm;
  params[ng++] = mom;
  // With the lag the ascent evaluates the extrapolated point twice in a row, the log-likelihood and
  // then the gradient, with only SetFixedEffects calls between (which write no parameter buffer).
  // A run computes both, so the second evaluation reuses the first run when the parameter buffers
  // and the buffer the deformed template was copied from are the same.
  const double *fe_src = tmpl, *def_src = tmpl;  // parameter buffers behind tmpl_fe and lm0
  const double *last_p[3] = {nullptr, nullptr, nullptr}, *last_def = nullptr;
  bool last_nograd = false;
  FgaEvaluate ev = [&](double *const *p, bool need_grad, double *terms, double *const *g, double *sq) -> int {
    int e = GBK_OK;
    bool reuse = lag && need_grad && last_nograd && def_src == last_def;
    for (int k = 0; k < ng; ++k) reuse = reuse && last_p[k] == p[k];
    for (int k = 0; k < ng; ++k) last_p[k] = p[k];
    last_def = def_src;
    last_nograd = !need_grad;
    if (!reuse) {
      if (gcp >= 0) e = c->cuda(cudaMemcpyAsync(a->cp, p[gcp], n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      // without the lag the evaluation deforms its own template; with it, lm0 holds the template
      // of the previous SetFixedEffects call (set_fixed below)
      if (!e && gt >= 0 && !lag)
        e = c->cuda(cudaMemcpyAsync(a->lm0, p[gt], m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e && gt >= 0) e = c->cuda(cudaMemcpyAsync(a->smooth, p[gt], m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e) e = c->cuda(cudaMemcpyAsync(a->mom, p[gm], nm * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e) e = a->run();
    }
    double out[3];
    if (!e) e = c->cuda(cudaMemcpyAsync(out, a->out, sizeof out, cudaMemcpyDeviceToHost, st), "read L");
    double h[3] = {0, 0, 0};
    if (!e && need_grad) {
      if (gcp >= 0) e = c->cuda(cudaMemcpyAsync(g[gcp], a->gcp, n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e && gt >= 0)
        e = c->cuda(cudaMemcpyAsync(g[gt], a->gtmpl, m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e) e = c->cuda(cudaMemcpyAsync(g[gm], a->gmom, nm * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e) e = c->cuda(dot_f64(st, a->gcp, a->gcp, n, sq_dev, 0), "norm");
      if (!e) e = c->cuda(dot_f64(st, a->smoothing > 0 ? a->gtmpl_l2 : a->gtmpl, a->gtmpl, m, sq_dev + 1, 0), "norm");
      if (!e) e = c->cuda(dot_f64(st, a->gmom, a->gmom, nm, sq_dev + 2, 0), "norm");
      if (!e) e = c->cuda(cudaMemcpyAsync(h, sq_dev, sizeof h, cudaMemcpyDeviceToHost, st), "read norms");
    }
    if (!e) e = c->cuda(cudaStreamSynchronize(st), "sync");
    if (!e) {
      terms[0] = out[1];
      terms[1] = out[2];
      if (need_grad) {
        if (gcp >= 0) sq[gcp] = h[0];
        if (gt >= 0) sq[gt] = h[1];
        sq[gm] = h[2];
      }
    }
    return e;
  };
  FgaOptions o;
  o.estimator = c->estimator;
  o.max_iterations = max_iterations;
  o.max_line_search = max_line_search;
  o.nb_iter_freeze = nb_iter_freeze;
  o.initial_step = initial_step;
  o.shrink = shrink;
  o.expand = expand;
  o.tolerance = tolerance;
  FgaResult res;
  // SetFixedEffects (AbstractAtlas.cxx:52-65): the template objects take the previous fixed-effect
  // template
  FgaSetFixed sf = [&](double *const *p) -> int {
    def_src = fe_src;
    fe_src = p[gt];
    int e = c->cuda(cudaMemcpyAsync(a->lm0, a->tmpl_fe, m * sizeof(double), cudaMemcpyDeviceToDevice, st), "lag");
    if (!e) e = c->cuda(cudaMemcpyAsync(a->tmpl_fe, p[gt], m * sizeof(double), cudaMemcpyDeviceToDevice, st), "lag");
    return e;
  };
  if (!rc) rc = fast_gradient_ascent(c, st, ng, sizes, params, o, ev, &res, nullptr, nullptr, lag ? sf : FgaSetFixed());
  // later steps deform and smooth over the final template
  if (!rc && optimize_template) rc = c->cuda(cudaMemcpyAsync(a->lm0, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc && optimize_template) rc = c->cuda(cudaMemcpyAsync(a->smooth, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  if (sq_dev) cudaFree(sq_dev);
  if (rc) return rc;
  std::copy(res.history.begin(), res.history.end(), history);
  *iterations = res.rows;
  if (info) {  // steps and squared norms per group (cp, template, momenta; 0 when frozen)
    for (int k = 0; k < 10; ++k) info[k] = 0.0;
    if (gcp >= 0) info[0] = res.step[gcp], info[5] = res.sq[gcp];
    if (gt >= 0) info[1] = res.step[gt], info[6] = res.sq[gt];
    info[2] = res.step[gm];
    info[7] = res.sq[gm];
    info[3] = res.tau;
    info[4] = res.freeze;
    info[8] = (double)res.evaluations;
    info[9] = res.stop;
  }
  return GBK_OK;
}

void gbk_atlas_destroy(gbk_atlas *a) {
  if (!a) return;
  cudaSetDevice(a->c->device);
  if (a->stream) cudaStreamSynchronize(a->stream);
  a->release();
  delete a;
}

}  // extern "C"
