// traj.cuh -- quantum-jump trajectory ensembles.
#pragma once

#include "ham.cuh"

namespace qd {

constexpr int kTrajMaxChan = 32;
constexpr int kTrajMaxObs = 16;

// path (may be null) receives 0 for the resident Taylor kernel, 1 for the batched Arnoldi steps,
// and path[1] the sparse products per trajectory step.
void traj_run(qd_ham* H, const qd_traj_desc& d, const double* psi0_host, double* obs_mean, double* obs_stderr,
              int64_t* jumps_total, double* timings, int* path);

}  // namespace qd
