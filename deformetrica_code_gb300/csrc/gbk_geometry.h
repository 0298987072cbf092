// A surface data term (currents or varifold) between a deformable mesh S and a fixed target T,
// with persistent device buffers so that evaluate() allocates nothing and can be captured in a
// CUDA graph. See gbk_geometry.cu for the formulation.
#pragma once

#include <vector>

#include "gbk_ctx.h"

namespace gbk {

struct SurfaceTerm {
  int kind = 0;  // 0 currents (OrientedSurfaceMesh / OrientedPolyLine), 1 varifold (NonOriented...)
  int d = 3;     // dimension
  int cell = 3;  // vertices per cell: 3 triangles (d = 3), 2 segments (d = 2 or 3)
  int dw = 3;    // cell weight columns: d (normals, tangents) or d(d+1)/2 (their tensors)
  double sigma = 1.0;
  long nv = 0, nf = 0, nv_t = 0, nf_t = 0;
  int *tris = nullptr, *tris_t = nullptr, *csr_ptr = nullptr, *csr_fc = nullptr;
  // source faces: centres, normals (n or n~), normal tensors, dual weights, pass outputs
  double *cs = nullptr, *ns = nullptr, *mns = nullptr, *ws = nullptr;
  double *kts = nullptr, *ktt = nullptr, *gs = nullptr, *gt = nullptr, *kt = nullptr, *gk = nullptr;
  // target faces
  double *ct = nullptr, *nt = nullptr, *mnt = nullptr, *wt = nullptr, *kttt = nullptr;
  double *scal = nullptr;  // [0] |T|^2, [1] |S|^2, [2] <S,T>
  std::vector<void *> owned;

  int init(gbk_ctx *c, int kind, int d, int cell, double sigma, long nv, long nf, const int *cells_host,
           long nv_t, long nf_t, const int *cells_t_host);
  int set_target(gbk_ctx *c, const double *pts_t);
  int evaluate(gbk_ctx *c, const double *pts_s, double *match_dev, double *grad_dev, double scale,
               int accumulate);
  void release();
};

void build_csr(long nv, long nf, int cell, const int *cells, std::vector<int> &ptr, std::vector<int> &fc);

}  // namespace gbk
