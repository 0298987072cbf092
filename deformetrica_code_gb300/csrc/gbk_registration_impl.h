// The registration object behind gbk_registration_* (one subject of DeterministicAtlas with a
// template of one or several objects), shared with the multi-object atlas, which drives one of
// them per subject.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "gbk_ctx.h"
#include "gbk_deform_impl.h"
#include "gbk_geometry.h"

// One template object: its data term against the subject's object, its first vertex among the
// template's points and its data sigma^2 (DeformableMultiObject, DeterministicAtlas.cxx:121-125).
struct RegObject {
  gbk::SurfaceTerm surf;
  long off = 0, nv = 0, nv_t = 0;
  double sigma2 = 1.0;
};

struct gbk_registration {
  gbk_ctx *c = nullptr;
  int d = 3, T = 2, heun = 1, use_graph = 1, steps = 0;
  long ncp = 0, nv = 0, nv_t = 0;  // control points, template points, target points (all objects)
  double sigma_def = 1;
  cudaStream_t stream = nullptr;
  bool own_stream = true;
  std::vector<RegObject> objs;
  std::vector<void *> owned;
  double *cp = nullptr, *mom = nullptr, *pos = nullptr, *momt = nullptr, *lm = nullptr, *lm0 = nullptr;
  double *theta = nullptr, *thetaT = nullptr, *xp = nullptr, *xm = nullptr;
  double *kp = nullptr, *greg = nullptr, *gcp = nullptr, *gmom = nullptr;
  // out: [L, L_data, L_reg, sum of matches, <K p, p>, -, -, -, match of object 0, 1, ...]
  double *out = nullptr, *sigma2_dev = nullptr, *tgt = nullptr;
  gbk::DeformScratch s;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long graph_launches = 0;

  // Pipelined iteration (pipeline = 1: the registrations of gbk_registration_create and the subjects
  // of the multi-object atlas).
  // The iteration is two chains of small dependent launches twice over: the flow of the template
  // points needs the shooting's step t only, and the control-point adjoint needs the landmark
  // adjoint's step t only. A helper context c2 (its own stream, split partials, tickets and packed
  // coordinates) runs the flow and the control-point adjoint one step behind, so the two chains'
  // launches overlap, and a second helper c3 runs each control-point adjoint update's landmark pass
  // beside its control-point pass. The helpers' kernel sums count into c's pair counters and report
  // into c's status word; they join the capture of `stream` through events, so the graph holds every
  // chain. The landmark terms are kept apart (s3) whether or not the iteration is pipelined.
  int pipeline = 0;
  gbk_ctx *c2 = nullptr, *c3 = nullptr;
  unsigned long long *c2_words = nullptr, *c3_words = nullptr;  // the helpers' own counter allocations
  gbk::DeformScratch s2;  // the helper chain's temporaries
  gbk::DeformScratch s3;  // the control-point adjoint's landmark terms (predictor va/vb, corrector vc/vd)
  // T - 1 shooting steps, T landmark-adjoint steps, 2 joins, 4 (T - 1) landmark-pass forks and joins
  std::vector<cudaEvent_t> ev;

  int alloc(void **p, size_t bytes);
  int enable_pipeline();
  void drop_helpers();
  int body();   // the whole iteration on `stream`, device pointers only
  int run();    // eager, then captured, then replayed
  void drop_graph();
  void release();
};

namespace gbk {

// Registrations run their iteration pipelined on three streams unless GBK_PIPELINE=0 (the value for
// gbk_registration::pipeline).
int pipeline_default();

// Creates a registration with nobj template objects: object k has kinds[k] (data_kind of
// gbk_registration_create), nv[k] template points (concatenated in tmpl_pts) and nf[k] cells
// (concatenated in cells, indices local to the object), its target's nv_t[k] points and nf_t[k]
// cells likewise, data kernel width sigma_data[k] and data sigma^2 data_sigma2[k]. With a non-null
// `stream` the registration runs on it instead of a stream of its own.
int registration_create(gbk_ctx *c, int d, long ncp, int nobj, const int *kinds, const long *nv,
                        const double *tmpl_pts, const long *nf, const int *cells, const long *nv_t,
                        const double *tgt_pts, const long *nf_t, const int *tgt_cells, const double *sigma_data,
                        const double *data_sigma2, int T, double sigma_def, int heun, cudaStream_t stream,
                        gbk_registration **out);

}  // namespace gbk
