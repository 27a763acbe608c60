// gauge_kernels.cuh -- launchers of the stout / force-chain kernels (gauge.cu).
#pragma once
#include <cuda_runtime.h>

namespace ost {
void ensure_ch_table(cudaStream_t st);
void launch_stout(const double2* u, double2* uout, double* qa, double2* stap, double rho, cudaStream_t st);
void launch_exp_times_conf(const double2* u, const double* qa, double2* uout, cudaStream_t st);
void launch_lambda(double* lam, const double2* sp, const double2* u, const double* qa, cudaStream_t st);
void launch_sigma(const double* lam, const double2* u, double2* s, const double* qa, double rho, cudaStream_t st);
void launch_force_outer(const double2* xs, const double2* ys, long vstride, int nshift, const double* coef_dev,
                        const double* ph, double2* pip, int with_phase, cudaStream_t st);
void launch_backfield(const double* ph, const double2* aux, double2* pip, cudaStream_t st);
void launch_conf_force_ta(const double2* u, const double2* sig, double* ip, cudaStream_t st);
}  // namespace ost
