// Device-pointer loop bodies of the deformation engine (gbk_deform.cu), shared with the
// registration and atlas objects.
#pragma once

#include "gbk_ctx.h"

namespace gbk {

struct DeformScratch {
  int *flag;  // "momenta below 1e-20" flag (device int)
  double *va;  // max(ncp, nlm) x d temporaries
  double *vb;
  double *vc;
  double *vd;
};

// Observations along the flow for the landmark adjoint (geodesic regression): n match gradients
// (device, nlm x d each) at increasing time indices (host). reference = 1 restates
// AdjointEquationsIntegrator.cxx:59-136 with jumps; 0 adds each gradient to theta at its index.
struct AdjointJumps {
  int n = 0;
  const int *times = nullptr;
  const double *const *grads = nullptr;
  int reference = 1;
};

// span = tn - t0: the time points are t0 + span k / (T - 1) (Diffeos::SetT0 / SetTN).
int shoot_device(gbk_ctx *c, int d, long ncp, const double *cp0, const double *mom0, int T,
                 double sigma, double *pos, double *mom, const DeformScratch &s, double span = 1.0);
int flow_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, int T,
                double sigma, long nlm, const double *lm0, int heun, double *lm,
                const DeformScratch &s, double span = 1.0);
// theta_final: the final condition without jumps (ignored when jumps has observations)
int adjoint_landmarks_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom,
                             int T, double sigma, long nlm, const double *lm,
                             const double *theta_final, int heun, double *theta,
                             const DeformScratch &s, double span = 1.0, const AdjointJumps *jumps = nullptr);
int update_at_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom,
                     const double *xp, const double *xm, long nlm, const double *lm,
                     const double *theta, double sigma, double *dpos, double *dmom);
int adjoint_diffeo_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, int T,
                          double sigma, long nlm, const double *lm, const double *theta, int heun,
                          double *xp, double *xm, const DeformScratch &s, double span = 1.0);

}  // namespace gbk
