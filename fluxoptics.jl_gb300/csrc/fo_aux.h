// Launchers of the elementwise / reduction kernels in fo_aux.cu.
#pragma once

#include <cuda_runtime.h>

namespace fo {

cudaError_t launch_as_h(float2* H, int fx_n, int fy_n, double dx, double dy, double lambda, double n0,
                        double z, double scale, cudaStream_t s);
cudaError_t launch_as_h_general(float2* H, int fx_n, int fy_n, double dx, double dy, double lambda, double n0,
                                double z, double scale, int mode, double theta_x, double theta_y, int track,
                                const double2* filter, cudaStream_t s, const float* zp = nullptr);
cudaError_t launch_as_h_z(float2* H, int fx_n, int fy_n, double dx, double dy, double lambda, double n0,
                          const float* z, double scale, cudaStream_t s);
int as_z_grad_blocks();
cudaError_t launch_as_z_grad(const float2* U, const float2* G, const float2* H, const int* h_index,
                             const float4* par, int mode, int track, int fx_n, int fy_n, double dx, double dy,
                             const float* z, int batch, int backward, double* partials, float* dz, cudaStream_t st);
cudaError_t launch_fourier_h(float2* H, int kind, const void* param, long long n, double scale, cudaStream_t s);
cudaError_t launch_fourier_grad(int kind, const void* param, const float2* U, const float2* A, void* grad,
                                long long npix, int batch, float s, cudaStream_t st);
cudaError_t launch_rs_h_spatial(float2* h, int nx, int ny, int px, int py, double dx, double dy,
                                double lambda, double z, double scale, cudaStream_t s);

cudaError_t launch_phase_fwd(float2* u, const float* phi, float2* saved, long long npix, int batch,
                             float s, cudaStream_t st);
cudaError_t launch_phase_bwd(float2* dv, const float* phi, const float2* saved, float* dphi,
                             long long npix, int batch, float s, cudaStream_t st);
cudaError_t launch_tea_fwd(float2* u, const float* h, const float4* coef, float2* saved, long long npix,
                           int batch, float s, cudaStream_t st);
cudaError_t launch_tea_bwd(float2* dv, const float* h, const float4* coef, const float2* saved, float* dh,
                           long long npix, int batch, float s, cudaStream_t st);
cudaError_t launch_mask_fwd(float2* u, const float2* m, float2* saved, long long npix, int batch,
                            int conj_m, cudaStream_t st);
cudaError_t launch_mask_bwd(float2* dv, const float2* m, const float2* saved, float2* dm,
                            long long npix, int batch, float s, cudaStream_t st);

int sid_partial_blocks(long long npix);
// loss[t] = fixed-order sum of partials[b * T + t] over b < nblocks
cudaError_t launch_sid_finalize(const float* partials, int nblocks, int T, float* loss, cudaStream_t st);
cudaError_t launch_sid_fwd(const float2* u, const float* target, const int* order, const int* offsets,
                           int T, long long npix, float* resid, float* partials, float* loss,
                           cudaStream_t st);
cudaError_t launch_sid_bwd(const float2* u, const float* resid, const int* tidx, const float* dc,
                           long long npix, int batch, float2* du, cudaStream_t st);

cudaError_t launch_fista(float* x, float* xk, float* newdx, const float* dx, long long n, float e,
                         double* t_state, cudaStream_t st, int clamp = 0,
                         float lo = 0.f, float hi = 0.f);
cudaError_t launch_clamp(float* x, long long n, float lo, float hi, cudaStream_t st);
// x <- s * conj(x) (conj != 0) or s * x, over n complex values
cudaError_t launch_conj_scale(float2* x, long long n, float s, int conj, cudaStream_t st);

size_t tv_state_bytes();
int tv_partial_blocks(long long n);
// TVProx on an nd-dimensional array (nd = 1..3, dims x fastest).
cudaError_t launch_tv(float* x, float* p, float* xk, float* yv, float* partials, void* state, int nd,
                      const int* dims, float lam, int n_iter, int isotropic, float e, cudaStream_t st,
                      double tol = 0.0, float* yprev = nullptr, float* maxima = nullptr);

}  // namespace fo
