// Elementwise and reduction kernels around the propagation passes: transfer
// functions (FP64), standalone modulators, the SquaredIntensityDifference metric,
// the Fista step, ClampProx and the TVProx dual iteration.
#include "fo_aux.h"
#include "fo_fft.cuh"

namespace fo {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(long long n, int threads = kThreads) {
  long long g = (n + threads - 1) / threads;
  return (unsigned)(g < 1 ? 1 : g);
}

__device__ __forceinline__ float2 cis_f(float a) {
  float s, c;
  sincosf(a, &s, &c);
  return make_float2(c, s);
}

// fftfreq(n, d)[k]: k/(n d) for k < ceil(n/2), (k-n)/(n d) otherwise.
__device__ __forceinline__ double fftfreq_d(int k, int n, double d) {
  const int h = (n + 1) / 2;
  return (double)(k < h ? k : k - n) / ((double)n * d);
}

// ---------------------------------------------------------------------------
// Transfer functions
// ---------------------------------------------------------------------------

// H[ky][kx] = cis(2 pi |z| sqrt(n0^2/lambda^2 - fx^2 - fy^2)) * scale, conj for z < 0;
// evanescent: exp(-2 pi |z| sqrt(fx^2 + fy^2 - n0^2/lambda^2)).
__global__ void as_h_kernel(float2* H, int fx_n, int fy_n, double dx, double dy, double f2,
                            double z, double scale) {
  const long long n = (long long)fx_n * fy_n;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(q % fx_n), ky = (int)(q / fx_n);
    const double fx = fftfreq_d(kx, fx_n, dx), fy = fftfreq_d(ky, fy_n, dy);
    const double arg = f2 - fx * fx - fy * fy;
    const double za = fabs(z);
    double re, im;
    if (arg >= 0.0) {
      const double ph = 2.0 * M_PI * za * sqrt(arg);
      sincos(ph, &im, &re);
    } else {
      re = exp(-2.0 * M_PI * za * sqrt(-arg));
      im = 0.0;
    }
    if (z < 0.0) im = -im;
    H[q] = make_float2((float)(re * scale), (float)(im * scale));
  }
}

// General angular-spectrum transfer function (angular_spectrum.jl:1-76), FP64:
//   mode 0 on axis : cis(2 pi z sqrt(1/lm^2 - fx^2 - fy^2))
//   mode 1 tilted  : cis(2 pi z (sqrt(1/lm^2 - (fx+f0x)^2 - (fy+f0y)^2) + off)), off = track ? (f0x fx + f0y fy) lm : 0
//   mode 2 paraxial: cis(-pi lm z ((fx+f0x)^2 + (fy+f0y)^2) - off + 2 pi z / lm), off = track ? 2 (f0x fx + f0y fy) : 0
// with lm = lambda / n0 and f0 = sin(theta) / lm; complex square root (evanescent
// components decay), times the optional filter values v (same layout) and `scale`.
// Modes 0 and 1 take conj(H(-z) v) for z < 0 (angular_spectrum.jl:9-12, 55-60), so the
// filter value is conjugated there too.  With zp the distance is read from device
// memory (ASPropZ, a trainable z) instead of `z`.
__global__ void as_h_general_kernel(float2* H, int fx_n, int fy_n, double dx, double dy, double lm, double z,
                                    double scale, int mode, double f0x, double f0y, int track,
                                    const double2* filter, const float* zp) {
  if (zp) z = (double)*zp;
  const long long n = (long long)fx_n * fy_n;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(q % fx_n), ky = (int)(q / fx_n);
    const double fx = fftfreq_d(kx, fx_n, dx), fy = fftfreq_d(ky, fy_n, dy);
    double re, im;
    if (mode == 2) {
      const double gx = fx + f0x, gy = fy + f0y;
      const double off = track ? 2.0 * (f0x * fx + f0y * fy) : 0.0;
      const double ph = -M_PI * lm * z * (gx * gx + gy * gy) - off + 2.0 * M_PI * z / lm;
      sincos(ph, &im, &re);
    } else {
      const double gx = mode == 1 ? fx + f0x : fx, gy = mode == 1 ? fy + f0y : fy;
      const double off = (mode == 1 && track) ? (f0x * fx + f0y * fy) * lm : 0.0;
      const double arg = 1.0 / (lm * lm) - gx * gx - gy * gy;
      const double za = fabs(z);
      // cis(2 pi za (sqrt(arg) + off)); sqrt(arg) = i sqrt(-arg) when arg < 0
      const double amp = arg >= 0.0 ? 1.0 : exp(-2.0 * M_PI * za * sqrt(-arg));
      const double ph = 2.0 * M_PI * za * ((arg >= 0.0 ? sqrt(arg) : 0.0) + off);
      double s, c;
      sincos(ph, &s, &c);
      re = amp * c;
      im = amp * s;
      if (z < 0.0) im = -im;
    }
    if (filter) {
      double2 f = filter[q];
      if (mode != 2 && z < 0.0) f.y = -f.y;
      const double r2 = re * f.x - im * f.y;
      im = re * f.y + im * f.x;
      re = r2;
    }
    H[q] = make_float2((float)(re * scale), (float)(im * scale));
  }
}

// On-axis transfer function with the distance read from device memory (ASPropZ,
// trainable z): as as_h_kernel, in FP64 from the float z.
__global__ void as_h_z_kernel(float2* H, int fx_n, int fy_n, double dx, double dy, double f2, const float* zp,
                              double scale) {
  const double z = (double)*zp;
  const long long n = (long long)fx_n * fy_n;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(q % fx_n), ky = (int)(q / fx_n);
    const double fx = fftfreq_d(kx, fx_n, dx), fy = fftfreq_d(ky, fy_n, dy);
    const double arg = f2 - fx * fx - fy * fy;
    const double za = fabs(z);
    double re, im;
    if (arg >= 0.0) {
      sincos(2.0 * M_PI * za * sqrt(arg), &im, &re);
    } else {
      re = exp(-2.0 * M_PI * za * sqrt(-arg));
      im = 0.0;
    }
    if (z < 0.0) im = -im;
    H[q] = make_float2((float)(re * scale), (float)(im * scale));
  }
}

// d loss / d z of ASPropZ: per block, sum over its frequency pixels k and the fields
// b of Re(U_b[k] conj(G_b[k]) dH_b[k]), conjugated for the Backward direction; U =
// FFT2(input), G = FFT2(adjoint at the output), H the stored table (which carries the
// 1/N of the inverse transform and the filter, constant in z).  dH/dz = i R H with the
// phase rate R of the table's kernel (mode as in as_h_general_kernel, g = f + f0):
//   modes 0 / 1: R = 2 pi (sqrt(complex(1/lm^2 - |g|^2)) + off), conjugated for z < 0,
//                off = track ? (f0x fx + f0y fy) lm : 0 (mode 1 only)
//   mode 2     : R = -pi lm |g|^2 + 2 pi / lm (the offset does not depend on z).
// par[b] = {1/lm, f0x, f0y, lm} of field b (f0 = 0 in mode 0).
__global__ void as_z_grad_partial_kernel(const float2* U, const float2* G, const float2* H, const int* h_index,
                                         const float4* par, int mode, int track, int fx_n, int fy_n, double dx,
                                         double dy, const float* zp, int batch, int backward, double* partials) {
  __shared__ double red[kThreads / 32];
  const long long npix = (long long)fx_n * fy_n;
  const bool zneg = *zp < 0.f;
  double acc = 0.0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npix;
       q += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(q % fx_n), ky = (int)(q / fx_n);
    const float fx = (float)fftfreq_d(kx, fx_n, dx), fy = (float)fftfreq_d(ky, fy_n, dy);
    float t = 0.f;
    for (int b = 0; b < batch; ++b) {
      const float4 pb = par[b];
      const float gx = fx + pb.y, gy = fy + pb.z;
      const float g2 = gx * gx + gy * gy;
      float2 rate;  // R
      if (mode == 2) {
        rate = make_float2(-3.14159265358979f * pb.w * g2 + 6.283185307179586f / pb.w, 0.f);
      } else {
        const float arg = pb.x * pb.x - g2;
        // sqrt(complex(arg)); conj for z < 0
        float2 kz = arg >= 0.f ? make_float2(sqrtf(arg), 0.f) : make_float2(0.f, sqrtf(-arg));
        if (zneg) kz.y = -kz.y;
        const float off = (mode == 1 && track) ? (pb.y * fx + pb.z * fy) * pb.w : 0.f;
        rate = make_float2(6.283185307179586f * (kz.x + off), 6.283185307179586f * kz.y);
      }
      float2 h = H[(long long)h_index[b] * npix + q];
      // dH = i R H
      float2 dh = cmul(make_float2(-rate.y, rate.x), h);
      if (backward) dh = cconj(dh);
      const long long o = (long long)b * npix + q;
      const float2 ug = cmul(U[o], cconj(G[o]));
      t += ug.x * dh.x - ug.y * dh.y;  // Re(U conj(G) dH)
    }
    acc += (double)t;
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) s += red[w];
    partials[blockIdx.x] = s;
  }
}

__global__ void as_z_grad_final_kernel(const double* partials, int nblk, float* dz) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += partials[b];
    *dz = (float)s;
  }
}

// Fourier-domain modulator multiplier: H = cis(phi) / N (phase) or m / N (mask);
// the Backward direction applies conj(H) in the column pass.
__global__ void fourier_h_kernel(float2* H, int kind, const void* param, long long n, float scale) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    float2 w;
    if (kind == 1) {
      float s, c;
      sincosf(reinterpret_cast<const float*>(param)[q], &s, &c);
      w = make_float2(c, s);
    } else {
      w = reinterpret_cast<const float2*>(param)[q];
    }
    H[q] = make_float2(w.x * scale, w.y * scale);
  }
}

// Gradient of a Fourier-domain modulator from the spectra U = FFT2(input) and
// A = FFT2(adjoint at the output), per frequency pixel over the batch in order:
// phase: s sum_b Im(cis(-s phi) A_b conj(U_b)); mask: sum_b conj_s(A_b conj(U_b))
// (the Phase and Mask gradients of phasemask.jl:115-150 and mask.jl:263-291 applied
// to the spectra, as FourierWrapper runs them, fourier/fourier_wrapper.jl:1-5).
__global__ void fourier_grad_kernel(int kind, const void* param, const float2* U, const float2* A, void* grad,
                                    long long npix, int batch, float s) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    if (kind == 1) {
      const float2 w = cis_f(-s * reinterpret_cast<const float*>(param)[p]);
      float acc = 0.f;
      for (int b = 0; b < batch; ++b) {
        const long long q = (long long)b * npix + p;
        const float2 du = cmul(A[q], w);
        const float2 u = U[q];
        acc += du.y * u.x - du.x * u.y;
      }
      reinterpret_cast<float*>(grad)[p] = s * acc;
    } else {
      float2 acc = make_float2(0.f, 0.f);
      for (int b = 0; b < batch; ++b) {
        const long long q = (long long)b * npix + p;
        float2 g = cmul(A[q], cconj(U[q]));
        if (s < 0.f) g = cconj(g);
        acc = cadd(acc, g);
      }
      reinterpret_cast<float2*>(grad)[p] = acc;
    }
  }
}

// Rayleigh-Sommerfeld impulse response on the circular (py x px) offset grid:
// offsets 0..n-1 at the start and -(n-1)..-1 at the end of each axis, zero between.
__global__ void rs_h_spatial_kernel(float2* h, int nx, int ny, int px, int py, double dx, double dy,
                                    double lambda, double z, double scale) {
  const long long n = (long long)px * py;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(q % px), iy = (int)(q / px);
    int ox, oy;
    bool ok = true;
    if (ix < nx) ox = ix; else if (ix > px - nx) ox = ix - px; else { ox = 0; ok = false; }
    if (iy < ny) oy = iy; else if (iy > py - ny) oy = iy - py; else { oy = 0; ok = false; }
    float2 out = make_float2(0.f, 0.f);
    if (ok) {
      const double x = ox * dx, y = oy * dy, za = fabs(z);
      const double k = 2.0 * M_PI / lambda;
      const double r = sqrt(x * x + y * y + za * za);
      const double nrm = dx * dy / (2.0 * M_PI);
      double s, c;
      sincos(k * r, &s, &c);
      // nrm * cis(k r)/r * (z/r) * (1/r - i k)
      const double a = nrm * za / (r * r);
      const double br = 1.0 / r, bi = -k;
      double re = a * (c * br - s * bi);
      double im = a * (c * bi + s * br);
      if (z < 0.0) im = -im;
      out = make_float2((float)(re * scale), (float)(im * scale));
    }
    h[q] = out;
  }
}

// ---------------------------------------------------------------------------
// Standalone modulators
// ---------------------------------------------------------------------------

__global__ void phase_fwd_kernel(float2* u, const float* phi, float2* saved, long long npix, int batch,
                                 float s) {
  const long long n = npix * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float2 x = u[q];
    if (saved) saved[q] = x;
    u[q] = cmul(x, cis_f(s * phi[q % npix]));
  }
}

__global__ void phase_bwd_kernel(float2* dv, const float* phi, const float2* saved, float* dphi,
                                 long long npix, int batch, float s) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    const float2 w = cis_f(-s * phi[p]);
    float acc = 0.f;
    for (int b = 0; b < batch; ++b) {
      const long long q = (long long)b * npix + p;
      const float2 du = cmul(dv[q], w);
      dv[q] = du;
      if (dphi) {
        const float2 u = saved[q];
        acc += du.y * u.x - du.x * u.y;
      }
    }
    if (dphi) dphi[p] = s * acc;
  }
}

// TeaDOE: field b is multiplied by r_b cis(s k_b h) (conj(r_b) for s < 0), with
// coef[b] = {k_b, Re r_b, Im r_b, 0} (modulators/tea_doe.jl:150-156).
__global__ void tea_fwd_kernel(float2* u, const float* h, const float4* coef, float2* saved, long long npix,
                               int batch, float s) {
  const long long n = npix * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(q / npix);
    const float4 c = coef[b];
    const float2 r = make_float2(c.y, s < 0.f ? -c.z : c.z);
    const float2 x = u[q];
    if (saved) saved[q] = x;
    u[q] = cmul(x, cmul(r, cis_f(s * c.x * h[q % npix])));
  }
}

// Adjoint: du_b = conj(r_b cis(s k_b h)) dv_b; dh = sum_b s k_b Im(du_b conj(u_saved_b)),
// one thread per pixel looping over the batch in order (tea_doe.jl:180-215).
__global__ void tea_bwd_kernel(float2* dv, const float* h, const float4* coef, const float2* saved, float* dh,
                               long long npix, int batch, float s) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    const float hp = h[p];
    float acc = 0.f;
    for (int b = 0; b < batch; ++b) {
      const float4 c = coef[b];
      const float2 r = make_float2(c.y, s < 0.f ? c.z : -c.z);  // conj of the forward amplitude
      const long long q = (long long)b * npix + p;
      const float2 du = cmul(dv[q], cmul(r, cis_f(-s * c.x * hp)));
      dv[q] = du;
      if (dh) {
        const float2 u = saved[q];
        acc = fmaf(s * c.x, du.y * u.x - du.x * u.y, acc);
      }
    }
    if (dh) dh[p] = acc;
  }
}

__global__ void mask_fwd_kernel(float2* u, const float2* m, float2* saved, long long npix, int batch,
                                int conj_m) {
  const long long n = npix * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float2 x = u[q];
    if (saved) saved[q] = x;
    float2 mm = m[q % npix];
    if (conj_m) mm = cconj(mm);
    u[q] = cmul(x, mm);
  }
}

__global__ void mask_bwd_kernel(float2* dv, const float2* m, const float2* saved, float2* dm,
                                long long npix, int batch, float s) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    float2 mm = m[p];
    if (s > 0.f) mm = cconj(mm);
    float2 acc = make_float2(0.f, 0.f);
    for (int b = 0; b < batch; ++b) {
      const long long q = (long long)b * npix + p;
      const float2 d = dv[q];
      if (dm) {
        float2 g = cmul(d, cconj(saved[q]));
        if (s < 0.f) g = cconj(g);
        acc = cadd(acc, g);
      }
      dv[q] = cmul(d, mm);
    }
    if (dm) dm[p] = acc;
  }
}

// ---------------------------------------------------------------------------
// SquaredIntensityDifference
// ---------------------------------------------------------------------------

template <int BS>
__device__ float block_sum(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  float r = 0.f;
  if (threadIdx.x < 32) {
    r = (threadIdx.x < BS / 32) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// One thread per pixel; fields visited target by target in the order of `order`
// (offsets[t]..offsets[t+1]).  Writes resid[t][p] = I_t - target_t and per-block
// partial sums of resid^2 (partials[block * T + t]).
__global__ void sid_fwd_kernel(const float2* u, const float* target, const int* order,
                               const int* offsets, int T, long long npix, float* resid,
                               float* partials) {
  __shared__ float red[kThreads / 32];
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool ok = p < npix;
  for (int t = 0; t < T; ++t) {
    float r2 = 0.f;
    if (ok) {
      float inten = 0.f;
      for (int f = offsets[t]; f < offsets[t + 1]; ++f) {
        const float2 x = u[(long long)order[f] * npix + p];
        inten = fmaf(x.x, x.x, fmaf(x.y, x.y, inten));
      }
      const float r = inten - target[(long long)t * npix + p];
      resid[(long long)t * npix + p] = r;
      r2 = r * r;
    }
    const float bs = block_sum<kThreads>(r2, red);
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * T + t] = bs;
  }
}

// loss[t] = sum over blocks of partials[block][t], fixed order, one CTA per t.
__global__ void sid_finalize_kernel(const float* partials, int nblocks, int T, float* loss) {
  __shared__ float red[kThreads / 32];
  const int t = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partials[(long long)b * T + t];
  const float s = block_sum<kThreads>((float)acc, red);
  if (threadIdx.x == 0) loss[t] = s;
}

__global__ void sid_bwd_kernel(const float2* u, const float* resid, const int* tidx, const float* dc,
                               long long npix, int batch, float2* du) {
  const long long n = npix * batch;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(q / npix);
    const long long p = q % npix;
    const int t = tidx[b];
    const float k = 4.f * (dc ? dc[t] : 1.f) * resid[(long long)t * npix + p];
    du[q] = cscale(u[q], k);
  }
}

// ---------------------------------------------------------------------------
// Fista / Clamp
// ---------------------------------------------------------------------------

// One Fista step, optionally followed by clamp(x, lo, hi).  beta comes from the FP64
// t state once per block (FP64 is a slow pipe on this part); four floats per thread
// and iteration where the arrays allow it.
__device__ __forceinline__ float fista_one(float xv, float xkv, float dxv, float e, float beta, float* nd_out) {
  const float nd = e * dxv - beta * (xv - xkv);
  *nd_out = nd;
  return xv - nd;
}

__global__ void fista_kernel(float* x, float* xk, float* newdx, const float* dx, long long n, float e,
                             const double* t_state, int clamp, float lo, float hi) {
  __shared__ float s_beta;
  if (threadIdx.x == 0) {
    const double t = *t_state;
    const double tn = (1.0 + sqrt(1.0 + 4.0 * t * t)) / 2.0;
    s_beta = (float)((t - 1.0) / tn);
  }
  __syncthreads();
  const float beta = s_beta;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const bool vec = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(xk) |
                     reinterpret_cast<uintptr_t>(dx) | reinterpret_cast<uintptr_t>(newdx)) & 15) == 0;
  const long long n4 = vec ? n / 4 : 0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n4; q += stride) {
    const float4 xv = reinterpret_cast<const float4*>(x)[q];
    const float4 kv = reinterpret_cast<const float4*>(xk)[q];
    const float4 dv = reinterpret_cast<const float4*>(dx)[q];
    float4 nd, xo;
    xo.x = fista_one(xv.x, kv.x, dv.x, e, beta, &nd.x);
    xo.y = fista_one(xv.y, kv.y, dv.y, e, beta, &nd.y);
    xo.z = fista_one(xv.z, kv.z, dv.z, e, beta, &nd.z);
    xo.w = fista_one(xv.w, kv.w, dv.w, e, beta, &nd.w);
    if (clamp) {
      xo.x = fminf(fmaxf(xo.x, lo), hi);
      xo.y = fminf(fmaxf(xo.y, lo), hi);
      xo.z = fminf(fmaxf(xo.z, lo), hi);
      xo.w = fminf(fmaxf(xo.w, lo), hi);
    }
    if (newdx) reinterpret_cast<float4*>(newdx)[q] = nd;
    reinterpret_cast<float4*>(xk)[q] = xv;
    reinterpret_cast<float4*>(x)[q] = xo;
  }
  for (long long q = 4 * n4 + blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += stride) {
    const float xv = x[q];
    float nd;
    float xo = fista_one(xv, xk[q], dx[q], e, beta, &nd);
    if (clamp) xo = fminf(fmaxf(xo, lo), hi);
    if (newdx) newdx[q] = nd;
    xk[q] = xv;
    x[q] = xo;
  }
}

__global__ void fista_t_kernel(double* t_state) {
  const double t = *t_state;
  *t_state = (1.0 + sqrt(1.0 + 4.0 * t * t)) / 2.0;
}

__global__ void clamp_kernel(float* x, long long n, float lo, float hi) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    x[q] = fminf(fmaxf(x[q], lo), hi);
}

// x <- s * conj(x) (conj != 0) or s * x
__global__ void conj_scale_kernel(float2* x, long long n, float s, int conj) {
  const float sy = conj ? -s : s;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float2 v = x[q];
    x[q] = make_float2(s * v.x, sy * v.y);
  }
}

// ---------------------------------------------------------------------------
// TVProx on 1-, 2- or 3-D arrays (x fastest, then y, then z).  p holds one dual
// slice per dimension (the forward differences along it).  The dual is used through
// a per-slice scale (the isotropic projection of the previous iteration), applied
// on read.
// ---------------------------------------------------------------------------

struct TvGrid {
  int nd;       // 1, 2 or 3
  int n[3];     // extents (x, y, z); unused ones are 1
  long long s[3];  // strides
  long long total;
};

struct TvState {  // device-resident scalars
  double t;        // Fista t of the dual iteration
  float beta;      // Fista beta of the next update
  float scale[3];  // per-slice projection factor of the current dual
  int done;        // the tolerance was met: the remaining iterations do nothing
};

__global__ void tv_init_kernel(float* p, float* xk, long long np, TvState* st) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < np;
       q += (long long)gridDim.x * blockDim.x) {
    p[q] = 0.f;
    xk[q] = 0.f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->t = 1.0;
    const double tn = (1.0 + sqrt(5.0)) / 2.0;
    st->beta = (float)((1.0 - 1.0) / tn);
    st->scale[0] = st->scale[1] = st->scale[2] = 1.f;
    st->done = 0;
  }
}

__device__ __forceinline__ void tv_coords(const TvGrid& g, long long q, int (&c)[3]) {
  c[0] = (int)(q % g.n[0]);
  const long long r = q / g.n[0];
  c[1] = (int)(r % g.n[1]);
  c[2] = (int)(r / g.n[1]);
}

// D^T of the reference (tv_prox.jl:43-59), on the scaled dual: the sum over the
// dimensions of p_i[c - e_i] - p_i[c], except that a point on the first plane of some
// dimension takes -p_J[c] of the highest such dimension J (the reference's boundary
// assignments, made in dimension order, overwrite one another).
__device__ __forceinline__ float tv_dt(const float* p, const float (&sc)[3], const TvGrid& g, long long q,
                                       const int (&c)[3]) {
  for (int i = g.nd - 1; i >= 0; --i)
    if (c[i] == 0) return -sc[i] * p[i * g.total + q];
  float v = 0.f;
  for (int i = 0; i < g.nd; ++i) {
    const float* pi = p + i * g.total;
    v += sc[i] * (pi[q - g.s[i]] - pi[q]);
  }
  return v;
}

// y = lam * D^T(p) - y0.  With a tolerance (yprev != NULL): per-block maxima of
// |y - y_prev| (y_prev: the previous iteration's y, zero before the first), and
// y_prev <- y.
__global__ void tv_dt_kernel(const float* p, const float* y0, float* yv, TvGrid g, float lam, const TvState* st,
                             float* yprev, float* maxima) {
  __shared__ float red[kThreads / 32];
  if (st->done) return;
  const float sc[3] = {st->scale[0], st->scale[1], st->scale[2]};
  float mx = 0.f;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.total;
       q += (long long)gridDim.x * blockDim.x) {
    int c[3];
    tv_coords(g, q, c);
    const float v = lam * tv_dt(p, sc, g, q, c) - y0[q];
    yv[q] = v;
    if (yprev) {
      mx = fmaxf(mx, fabsf(yprev[q] - v));
      yprev[q] = v;
    }
  }
  if (yprev) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      float m = 0.f;
      for (int w = 0; w < kThreads / 32; ++w) m = fmaxf(m, red[w]);
      maxima[blockIdx.x] = m;
    }
  }
}

// The tolerance test of the iteration: max |y - y_prev| < tol stops it before its
// dual update (tv_prox.jl:158-166).
__global__ void tv_check_kernel(const float* maxima, int nblocks, double tol, TvState* st) {
  __shared__ float red[kThreads / 32];
  if (st->done) return;
  float mx = 0.f;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) mx = fmaxf(mx, maxima[b]);
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f;
    for (int w = 0; w < kThreads / 32; ++w) m = fmaxf(m, red[w]);
    if ((double)m < tol) st->done = 1;
  }
}

// dp = D(y); Fista on the (scaled) dual; per-block partial sums of p^2 per slice
// (isotropic) or clamp to [-1, 1] (anisotropic).
__global__ void tv_step_kernel(float* p, float* xk, const float* yv, TvGrid g, float e, const TvState* st,
                               int isotropic, float* partials) {
  __shared__ float red[kThreads / 32];
  if (st->done) return;
  const float beta = st->beta;
  float ss[3] = {0.f, 0.f, 0.f};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.total;
       q += (long long)gridDim.x * blockDim.x) {
    int c[3];
    tv_coords(g, q, c);
    const float yc = yv[q];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (i >= g.nd) break;
      const float d = (c[i] < g.n[i] - 1) ? yv[q + g.s[i]] - yc : 0.f;
      const long long qi = q + i * g.total;
      const float pv = p[qi] * st->scale[i];
      const float nd = e * d - beta * (pv - xk[qi]);
      xk[qi] = pv;
      float pn = pv - nd;
      if (!isotropic) pn = fminf(fmaxf(pn, -1.f), 1.f);
      p[qi] = pn;
      ss[i] = fmaf(pn, pn, ss[i]);
    }
  }
  if (isotropic) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (i >= g.nd) break;
      const float b = block_sum<kThreads>(ss[i], red);
      if (threadIdx.x == 0) partials[blockIdx.x * 3 + i] = b;
    }
  }
}

// Per-slice norms -> projection scale; Fista t/beta for the next update.
__global__ void tv_norm_kernel(const float* partials, int nblocks, int nd, int isotropic, TvState* st) {
  __shared__ float red[kThreads / 32];
  if (st->done) return;
  float sc[3] = {1.f, 1.f, 1.f};
  if (isotropic) {
    for (int i = 0; i < nd; ++i) {
      double acc = 0.0;
      for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partials[b * 3 + i];
      const float s = block_sum<kThreads>((float)acc, red);
      if (threadIdx.x == 0) {
        const float nrm = sqrtf(s);
        sc[i] = nrm > 1.f ? 1.f / nrm : 1.f;
      }
    }
  }
  if (threadIdx.x == 0) {
    st->scale[0] = sc[0];
    st->scale[1] = sc[1];
    st->scale[2] = sc[2];
    const double t = (1.0 + sqrt(1.0 + 4.0 * st->t * st->t)) / 2.0;  // t after this update
    const double tn = (1.0 + sqrt(1.0 + 4.0 * t * t)) / 2.0;
    st->t = t;
    st->beta = (float)((t - 1.0) / tn);
  }
}

// y0 -= lam * D^T(p)
__global__ void tv_final_kernel(const float* p, float* y0, TvGrid g, float lam, const TvState* st) {
  const float sc[3] = {st->scale[0], st->scale[1], st->scale[2]};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.total;
       q += (long long)gridDim.x * blockDim.x) {
    int c[3];
    tv_coords(g, q, c);
    y0[q] -= lam * tv_dt(p, sc, g, q, c);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------

static unsigned capped_grid(long long n) {
  long long g = (n + kThreads - 1) / kThreads;
  if (g > 152LL * 32) g = 152LL * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

cudaError_t launch_as_h(float2* H, int fx_n, int fy_n, double dx, double dy, double lambda, double n0,
                        double z, double scale, cudaStream_t s) {
  const double lm = lambda / n0;
  as_h_kernel<<<capped_grid((long long)fx_n * fy_n), kThreads, 0, s>>>(H, fx_n, fy_n, dx, dy,
                                                                       1.0 / (lm * lm), z, scale);
  return cudaGetLastError();
}

cudaError_t launch_as_h_general(float2* H, int fx_n, int fy_n, double dx, double dy, double lambda, double n0,
                                double z, double scale, int mode, double theta_x, double theta_y, int track,
                                const double2* filter, cudaStream_t s, const float* zp) {
  const double lm = lambda / n0;
  as_h_general_kernel<<<capped_grid((long long)fx_n * fy_n), kThreads, 0, s>>>(
      H, fx_n, fy_n, dx, dy, lm, z, scale, mode, sin(theta_x) / lm, sin(theta_y) / lm, track, filter, zp);
  return cudaGetLastError();
}

cudaError_t launch_as_h_z(float2* H, int fx_n, int fy_n, double dx, double dy, double lambda, double n0,
                          const float* z, double scale, cudaStream_t s) {
  const double lm = lambda / n0;
  as_h_z_kernel<<<capped_grid((long long)fx_n * fy_n), kThreads, 0, s>>>(H, fx_n, fy_n, dx, dy, 1.0 / (lm * lm), z,
                                                                        scale);
  return cudaGetLastError();
}

int as_z_grad_blocks() { return 304; }

cudaError_t launch_as_z_grad(const float2* U, const float2* G, const float2* H, const int* h_index,
                             const float4* par, int mode, int track, int fx_n, int fy_n, double dx, double dy,
                             const float* z, int batch, int backward, double* partials, float* dz, cudaStream_t st) {
  as_z_grad_partial_kernel<<<as_z_grad_blocks(), kThreads, 0, st>>>(U, G, H, h_index, par, mode, track, fx_n, fy_n,
                                                                   dx, dy, z, batch, backward, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  as_z_grad_final_kernel<<<1, 32, 0, st>>>(partials, as_z_grad_blocks(), dz);
  return cudaGetLastError();
}

cudaError_t launch_fourier_h(float2* H, int kind, const void* param, long long n, double scale, cudaStream_t s) {
  fourier_h_kernel<<<capped_grid(n), kThreads, 0, s>>>(H, kind, param, n, (float)scale);
  return cudaGetLastError();
}

cudaError_t launch_fourier_grad(int kind, const void* param, const float2* U, const float2* A, void* grad,
                                long long npix, int batch, float s, cudaStream_t st) {
  fourier_grad_kernel<<<capped_grid(npix), kThreads, 0, st>>>(kind, param, U, A, grad, npix, batch, s);
  return cudaGetLastError();
}

cudaError_t launch_rs_h_spatial(float2* h, int nx, int ny, int px, int py, double dx, double dy,
                                double lambda, double z, double scale, cudaStream_t s) {
  rs_h_spatial_kernel<<<capped_grid((long long)px * py), kThreads, 0, s>>>(h, nx, ny, px, py, dx, dy,
                                                                           lambda, z, scale);
  return cudaGetLastError();
}

cudaError_t launch_phase_fwd(float2* u, const float* phi, float2* saved, long long npix, int batch,
                             float s, cudaStream_t st) {
  phase_fwd_kernel<<<capped_grid(npix * batch), kThreads, 0, st>>>(u, phi, saved, npix, batch, s);
  return cudaGetLastError();
}

cudaError_t launch_phase_bwd(float2* dv, const float* phi, const float2* saved, float* dphi,
                             long long npix, int batch, float s, cudaStream_t st) {
  phase_bwd_kernel<<<capped_grid(npix), kThreads, 0, st>>>(dv, phi, saved, dphi, npix, batch, s);
  return cudaGetLastError();
}

cudaError_t launch_tea_fwd(float2* u, const float* h, const float4* coef, float2* saved, long long npix,
                           int batch, float s, cudaStream_t st) {
  tea_fwd_kernel<<<capped_grid(npix * batch), kThreads, 0, st>>>(u, h, coef, saved, npix, batch, s);
  return cudaGetLastError();
}

cudaError_t launch_tea_bwd(float2* dv, const float* h, const float4* coef, const float2* saved, float* dh,
                           long long npix, int batch, float s, cudaStream_t st) {
  tea_bwd_kernel<<<capped_grid(npix), kThreads, 0, st>>>(dv, h, coef, saved, dh, npix, batch, s);
  return cudaGetLastError();
}

cudaError_t launch_mask_fwd(float2* u, const float2* m, float2* saved, long long npix, int batch,
                            int conj_m, cudaStream_t st) {
  mask_fwd_kernel<<<capped_grid(npix * batch), kThreads, 0, st>>>(u, m, saved, npix, batch, conj_m);
  return cudaGetLastError();
}

cudaError_t launch_mask_bwd(float2* dv, const float2* m, const float2* saved, float2* dm,
                            long long npix, int batch, float s, cudaStream_t st) {
  mask_bwd_kernel<<<capped_grid(npix), kThreads, 0, st>>>(dv, m, saved, dm, npix, batch, s);
  return cudaGetLastError();
}

int sid_partial_blocks(long long npix) { return (int)grid_for(npix); }

cudaError_t launch_sid_finalize(const float* partials, int nblocks, int T, float* loss, cudaStream_t st) {
  sid_finalize_kernel<<<T, kThreads, 0, st>>>(partials, nblocks, T, loss);
  return cudaGetLastError();
}

cudaError_t launch_sid_fwd(const float2* u, const float* target, const int* order, const int* offsets,
                           int T, long long npix, float* resid, float* partials, float* loss,
                           cudaStream_t st) {
  const int nb = sid_partial_blocks(npix);
  sid_fwd_kernel<<<nb, kThreads, 0, st>>>(u, target, order, offsets, T, npix, resid, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sid_finalize_kernel<<<T, kThreads, 0, st>>>(partials, nb, T, loss);
  return cudaGetLastError();
}

cudaError_t launch_sid_bwd(const float2* u, const float* resid, const int* tidx, const float* dc,
                           long long npix, int batch, float2* du, cudaStream_t st) {
  sid_bwd_kernel<<<capped_grid(npix * batch), kThreads, 0, st>>>(u, resid, tidx, dc, npix, batch, du);
  return cudaGetLastError();
}

cudaError_t launch_fista(float* x, float* xk, float* newdx, const float* dx, long long n, float e,
                         double* t_state, cudaStream_t st, int clamp,
                         float lo, float hi) {
  fista_kernel<<<capped_grid((n + 3) / 4), kThreads, 0, st>>>(x, xk, newdx, dx, n, e, t_state, clamp, lo, hi);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  fista_t_kernel<<<1, 1, 0, st>>>(t_state);
  return cudaGetLastError();
}

cudaError_t launch_clamp(float* x, long long n, float lo, float hi, cudaStream_t st) {
  clamp_kernel<<<capped_grid(n), kThreads, 0, st>>>(x, n, lo, hi);
  return cudaGetLastError();
}

cudaError_t launch_conj_scale(float2* x, long long n, float s, int conj, cudaStream_t st) {
  conj_scale_kernel<<<capped_grid(n), kThreads, 0, st>>>(x, n, s, conj);
  return cudaGetLastError();
}

size_t tv_state_bytes() { return sizeof(TvState); }
int tv_partial_blocks(long long n) { return (int)capped_grid(n); }

cudaError_t launch_tv(float* x, float* p, float* xk, float* yv, float* partials, void* state, int nd,
                      const int* dims, float lam, int n_iter, int isotropic, float e, cudaStream_t st, double tol,
                      float* yprev, float* maxima) {
  TvGrid g;
  g.nd = nd;
  g.total = 1;
  for (int i = 0; i < 3; ++i) {
    g.n[i] = i < nd ? dims[i] : 1;
    g.s[i] = g.total;
    g.total *= g.n[i];
  }
  const long long n = g.total;
  TvState* s = reinterpret_cast<TvState*>(state);
  const unsigned blocks = capped_grid(n);
  const bool use_tol = tol > 0.0 && yprev && maxima;
  tv_init_kernel<<<capped_grid(nd * n), kThreads, 0, st>>>(p, xk, nd * n, s);
  if (use_tol) {
    cudaError_t e0 = cudaMemsetAsync(yprev, 0, sizeof(float) * n, st);
    if (e0 != cudaSuccess) return e0;
  }
  for (int it = 0; it < n_iter; ++it) {
    tv_dt_kernel<<<blocks, kThreads, 0, st>>>(p, x, yv, g, lam, s, use_tol ? yprev : nullptr, maxima);
    if (use_tol) tv_check_kernel<<<1, kThreads, 0, st>>>(maxima, (int)blocks, tol, s);
    tv_step_kernel<<<blocks, kThreads, 0, st>>>(p, xk, yv, g, e, s, isotropic, partials);
    tv_norm_kernel<<<1, kThreads, 0, st>>>(partials, (int)blocks, nd, isotropic, s);
  }
  tv_final_kernel<<<blocks, kThreads, 0, st>>>(p, x, g, lam, s);
  return cudaGetLastError();
}

}  // namespace fo
