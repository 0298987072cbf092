// A data term between a deformable object S and a fixed target T (currents, varifold, weighted
// point cloud, volume mesh, landmarks), with persistent device buffers so that evaluate()
// allocates nothing and can be captured in a CUDA graph. See gbk_geometry.cu for the formulation.
#pragma once

#include <vector>

#include "gbk_ctx.h"

namespace gbk {

struct SurfaceTerm {
  // 0 currents (OrientedSurfaceMesh / OrientedPolyLine), 1 varifold (NonOriented...), 2 scalar
  // measure (PointCloud: cell 1; OrientedVolumeMesh: cell d + 1), 3 landmarks (cell 1)
  int kind = 0;
  int d = 3;     // dimension
  int cell = 3;  // vertices per cell: 3 triangles (d = 3), 2 segments, d + 1 simplices, 1 points
  int dw = 3;    // cell weight columns: d (normals, tangents), d(d+1)/2 (their tensors), 1 (measures)
  int exact = 0; // GBK_GRADIENT_EXACT for the measure terms
  double sigma = 1.0;
  long nv = 0, nf = 0, nv_t = 0, nf_t = 0;
  int *tris = nullptr, *tris_t = nullptr, *csr_ptr = nullptr, *csr_fc = nullptr;
  // source faces: centres, normals (n or n~), normal tensors, dual weights, pass outputs
  double *cs = nullptr, *ns = nullptr, *mns = nullptr, *ws = nullptr;
  double *kts = nullptr, *ktt = nullptr, *gs = nullptr, *gt = nullptr, *kt = nullptr, *gk = nullptr;
  // target faces
  double *ct = nullptr, *nt = nullptr, *mnt = nullptr, *wt = nullptr, *kttt = nullptr;
  double *sg = nullptr;    // sign of each volume cell's determinant
  double *scal = nullptr;  // [0] |T|^2, [1] |S|^2, [2] <S,T>
  const double *tgt = nullptr;  // the target points of the last set_target
  std::vector<void *> owned;

  // cells_host / cells_t_host may be null for cell 1 (points: nf = nv); w_host / w_t_host are
  // the point weights of a point cloud (null = unit weights)
  int init(gbk_ctx *c, int kind, int d, int cell, double sigma, long nv, long nf, const int *cells_host,
           long nv_t, long nf_t, const int *cells_t_host, const double *w_host = nullptr,
           const double *w_t_host = nullptr);
  // replaces the point weights of a point cloud (device or host; null keeps them) and recomputes
  // the target norm from the last target
  int set_weights(gbk_ctx *c, const double *w, const double *w_t);
  int set_target(gbk_ctx *c, const double *pts_t);
  int evaluate(gbk_ctx *c, const double *pts_s, double *match_dev, double *grad_dev, double scale,
               int accumulate);
  void release();
};

void build_csr(long nv, long nf, int cell, const int *cells, std::vector<int> &ptr, std::vector<int> &fc);

}  // namespace gbk
