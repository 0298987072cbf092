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
//
// Two loops may run on two streams one step apart (the registration's pipelined iteration): the
// producer records step_done[k] on its stream after step k, the consumer's stream waits on
// wait_step[k] before its step k (and on wait_step of its first step before anything else). Steps are
// indexed by their t: shooting and flow t = 0 .. T-2 (the flow's step t reads the shooting's
// positions and momenta at t and t + 1), the adjoints t = T-1 .. 1 (the parameter adjoint's step t
// reads theta at t and t - 1, which the landmark adjoint's step t writes).
// zero_tail = false leaves the zeroing of mom[t >= 1] for nearly zero momenta to the caller (after
// a flow that reads mom has finished; its results do not depend on them then).
int shoot_device(gbk_ctx *c, int d, long ncp, const double *cp0, const double *mom0, int T,
                 double sigma, double *pos, double *mom, const DeformScratch &s, double span = 1.0,
                 const cudaEvent_t *step_done = nullptr, bool zero_tail = true);
int zero_tail_device(gbk_ctx *c, int d, long ncp, int T, double *mom, const DeformScratch &s);
int flow_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, int T,
                double sigma, long nlm, const double *lm0, int heun, double *lm,
                const DeformScratch &s, double span = 1.0, const cudaEvent_t *wait_step = nullptr);
// theta_final: the final condition without jumps (ignored when jumps has observations)
int adjoint_landmarks_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom,
                             int T, double sigma, long nlm, const double *lm,
                             const double *theta_final, int heun, double *theta,
                             const DeformScratch &s, double span = 1.0, const AdjointJumps *jumps = nullptr,
                             const cudaEvent_t *step_done = nullptr);
int update_at_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom,
                     const double *xp, const double *xm, long nlm, const double *lm,
                     const double *theta, double sigma, double *dpos, double *dmom);
// The control-point adjoint's landmark terms (dXi1, dXi2 of ComputeUpdateAt) kept apart from its
// control-point terms: the landmark pass writes s.va / s.vb (predictor) and s.vc / s.vd (corrector),
// which the Euler and Heun updates add in. With ctx set, the landmark pass runs on that context's
// stream concurrently with the control-point pass (events ev[4 (T-1-t) .. +3] fork and join the two
// passes of step t); with ctx null, on the same stream (same results bit for bit).
struct LandmarkSplit {
  gbk_ctx *ctx = nullptr;
  DeformScratch s{};
  const cudaEvent_t *ev = nullptr;
};
int adjoint_diffeo_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, int T,
                          double sigma, long nlm, const double *lm, const double *theta, int heun,
                          double *xp, double *xm, const DeformScratch &s, double span = 1.0,
                          const cudaEvent_t *wait_step = nullptr, const LandmarkSplit *split = nullptr);

}  // namespace gbk
