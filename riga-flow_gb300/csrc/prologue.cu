// prologue.cu — the FP64 device prologue of a pricing request.
//
// * calibrate_kernel: one CTA per Dupire surface.  Natural-spline fit of each tenor's smile in
//   log-moneyness, total-variance Dupire on the dense log-strike axis, clamp to [0.10, 3.00]
//   (crates/riga-market/src/lib.rs:125-299).  Writes the FP64 grid the parity kernel reads and
//   the (v, dv) FP32 pairs the production kernel interpolates.
// * cholesky_kernel: one thread per scenario.  Jacobi minimum eigenvalue, diagonal-loading PSD
//   clamp and Cholesky–Banachiewicz (crates/riga-market/src/correlation.rs:95-168), in place on
//   the scenario's correlation block; cholesky_big_kernel: the same for a book's universe.
// Compiled with -fmad=false so the FP64 arithmetic rounds like the reference's.  The calibration's
// logarithms and exponentials (the log-strike axis, the forwards, the log-moneyness of every
// strike and grid node: about n_t * (n_k + gx) values, independent of the paths) are evaluated on
// the host with the platform libm — the functions the reference's f64::ln / f64::exp call — and
// read here from CalibJob::ax, so a grid is bit-identical to the reference's calibration.  The
// spline and Dupire arithmetic, which amplifies a last-ulp change of any of those inputs about a
// million-fold, runs here in FP64.
#include "rg_internal.h"

namespace rg {

// Natural-spline second derivatives by the Thomas algorithm (riga-market/src/lib.rs:125-176).
__device__ static void spline_y2(const double* x, const double* y, int n, double* y2, double* h,
                                 double* cp, double* dp) {
  for (int i = 0; i < n; ++i) y2[i] = 0.0;
  if (n < 3) return;
  bool bad = false;
  for (int i = 0; i < n - 1; ++i) {
    h[i] = x[i + 1] - x[i];
    if (h[i] <= 0.0) bad = true;
  }
  for (int i = 0; i < n; ++i)
    if (!isfinite(y[i])) bad = true;
  if (bad) return;
  // b: diagonal; a/c: sub/super diagonals; d: right-hand side (computed inline)
  auto b = [&](int i) { return (i == 0 || i == n - 1) ? 1.0 : 2.0 * (h[i - 1] + h[i]); };
  auto a = [&](int i) { return i < n - 1 ? h[i] : 0.0; };
  auto c = [&](int i) { return i + 1 < n - 1 ? h[i + 1] : 0.0; };
  auto d = [&](int i) {
    return (i == 0 || i == n - 1) ? 0.0 : 6.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1]);
  };
  cp[0] = c(0) / b(0);
  dp[0] = d(0) / b(0);
  for (int i = 1; i < n; ++i) {
    double m = b(i) - a(i) * cp[i - 1];
    if (fabs(m) < 1e-300) m = 1e-300;
    cp[i] = c(i) / m;
    dp[i] = (d(i) - a(i) * dp[i - 1]) / m;
  }
  y2[n - 1] = dp[n - 1];
  for (int i = n - 2; i >= 0; --i) y2[i] = dp[i] - cp[i] * y2[i + 1];
}

// Spline value and derivatives with the reference's term placement (lib.rs:178-203).
__device__ static void spline_at(double p, const double* x, const double* y, const double* y2, int n,
                                 double* f, double* f1, double* f2) {
  int seg = 0;
  while (seg + 1 < n - 1 && p > x[seg + 1]) ++seg;
  double h = x[seg + 1] - x[seg];
  double t = (p - x[seg]) / h;
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  double omt = 1.0 - t;
  *f = (1.0 - t) * y[seg] + t * y[seg + 1] +
       (h * h / 6.0) * ((t * t * t - t) * y2[seg] + (omt * (omt * omt) - (1.0 - t)) * y2[seg + 1]);
  *f1 = (y[seg + 1] - y[seg] +
         (h * h / 6.0) * ((3.0 * t * t - 1.0) * y2[seg] - (3.0 * (1.0 - t) * (1.0 - t) - 1.0) * y2[seg + 1])) /
        h;
  *f2 = (1.0 - t) * y2[seg + 1] + t * y2[seg];
}

__global__ void calibrate_kernel(const CalibJob* __restrict__ jobs) {
  const CalibJob J = jobs[blockIdx.x];
  const int nt = J.n_t, nk = J.n_k, gx = J.gx;
  if (J.cache_src) {
    // a resident surface calibrated by an earlier call from the same inputs
    const double* sv = J.cache_src;
    const double* sl = sv + (size_t)nt * gx;
    const float2* sf = reinterpret_cast<const float2*>(sl + gx);
    for (int c = threadIdx.x; c < nt * gx; c += blockDim.x) {
      J.out_v[c] = sv[c];
      J.out_vf[c] = sf[c];
    }
    for (int i = threadIdx.x; i < gx; i += blockDim.x) J.out_logs[i] = sl[i];
    return;
  }
  double* w = J.scratch;
  double* wx = w + nt * gx;
  double* wxx = wx + nt * gx;
  double* xa = wxx + nt * gx;
  double* xj = xa + nt * gx + gx;             // nt * nk (after gx spare doubles)
  double* y2 = xj + nt * nk;                  // nt * nk
  double* tmp = y2 + nt * nk;                 // 3 * nt * nk (h, cp, dp)
  double* yv = tmp + 3 * nt * nk;             // nt * nk shifted implied vols
  const double* ax_logs = J.ax;               // gx
  const double* ax_xj = ax_logs + gx;         // nt * nk
  const double* ax_xd = ax_xj + nt * nk;      // nt * gx
  for (int i = threadIdx.x; i < gx; i += blockDim.x) J.out_logs[i] = ax_logs[i];
  for (int i = threadIdx.x; i < nt * nk; i += blockDim.x) {
    yv[i] = J.vols[i] + J.shift;
    xj[i] = ax_xj[i];
  }
  __syncthreads();
  // one thread per tenor: the spline solve on the log-moneyness nodes
  for (int k = threadIdx.x; k < nt; k += blockDim.x)
    spline_y2(xj + k * nk, yv + k * nk, nk, y2 + k * nk, tmp + 3 * k * nk, tmp + 3 * k * nk + nk,
              tmp + 3 * k * nk + 2 * nk);
  __syncthreads();
  for (int c = threadIdx.x; c < nt * gx; c += blockDim.x) {
    int k = c / gx;
    double tk = J.mats[k];
    const double* xk = xj + k * nk;
    double x_lo = xk[0], x_hi = xk[nk - 1];
    double xd = ax_xd[c];
    xd = xd < x_lo ? x_lo : (xd > x_hi ? x_hi : xd);
    double sg, s1, s2;
    if (nk >= 2) {
      spline_at(xd, xk, yv + k * nk, y2 + k * nk, nk, &sg, &s1, &s2);
    } else {
      sg = yv[k * nk];
      s1 = 0.0;
      s2 = 0.0;
    }
    w[c] = sg * sg * tk;
    wx[c] = 2.0 * sg * tk * s1;
    wxx[c] = 2.0 * tk * (s1 * s1 + sg * s2);
    xa[c] = xd;
  }
  __syncthreads();
  const double* T = J.mats;
  const double lo2 = 0.10 * 0.10, hi2 = 3.00 * 3.00;  // LV_CLAMP_LO/HI, lib.rs:30-32
  for (int c = threadIdx.x; c < nt * gx; c += blockDim.x) {
    int k = c / gx, i = c % gx;
    double dw;
    if (nt == 1) {
      dw = w[i] / (T[0] > 1e-9 ? T[0] : 1e-9);
    } else if (k == 0) {
      double sp = T[1] - T[0];
      dw = (w[gx + i] - w[i]) / (sp > 1e-9 ? sp : 1e-9);
    } else if (k == nt - 1) {
      double sp = T[nt - 1] - T[nt - 2];
      dw = (w[(nt - 1) * gx + i] - w[(nt - 2) * gx + i]) / (sp > 1e-9 ? sp : 1e-9);
    } else {
      double sp = T[k + 1] - T[k - 1];
      dw = (w[(k + 1) * gx + i] - w[(k - 1) * gx + i]) / (sp > 1e-9 ? sp : 1e-9);
    }
    double ww = w[c] > 1e-12 ? w[c] : 1e-12;
    double denom = 1.0 - (xa[c] / ww) * wx[c] + 0.25 * (-0.25 - 1.0 / ww) * wx[c] * wx[c] + 0.5 * wxx[c];
    double lv2 = (isfinite(denom) && fabs(denom) > 1e-12) ? dw / denom : lo2;
    lv2 = lv2 < lo2 ? lo2 : (lv2 > hi2 ? hi2 : lv2);
    J.out_v[c] = sqrt(lv2);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nt * gx; c += blockDim.x) {
    int i = c % gx;
    double v = J.out_v[c];
    double dv = i + 1 < gx ? J.out_v[c + 1] - v : 0.0;
    J.out_vf[c] = make_float2((float)v, (float)dv);
  }
  if (J.cache_dst) {
    __syncthreads();
    double* dv = J.cache_dst;
    double* dl = dv + (size_t)nt * gx;
    float2* df = reinterpret_cast<float2*>(dl + gx);
    for (int c = threadIdx.x; c < nt * gx; c += blockDim.x) {
      dv[c] = J.out_v[c];
      df[c] = J.out_vf[c];
    }
    for (int i = threadIdx.x; i < gx; i += blockDim.x) dl[i] = J.out_logs[i];
  }
}

// One CTA per (surface, step): the FP64 row sigma(step·dt, ·) of the surface, linear in tenor
// (riga-market/src/lib.rs:345-364), stored as FP32 lines of its cells in the grid position.
__global__ void lvrows_kernel(const double* __restrict__ lv_v, const int32_t* __restrict__ cell_off,
                              const int32_t* __restrict__ surf_asset, const int2* __restrict__ lv_ti,
                              const double* __restrict__ lv_tw, int T, int gx, float2* __restrict__ rows) {
  const int sfc = blockIdx.x, t = blockIdx.y;
  const int f = surf_asset[sfc];
  const int2 ti = lv_ti[f * T + t];
  const double wt = lv_tw[f * T + t];
  const double* v0 = lv_v + cell_off[sfc] + ti.x * gx;
  const double* v1 = lv_v + cell_off[sfc] + ti.y * gx;
  float2* out = rows + ((size_t)sfc * T + t) * gx;
  // cell j as a line in the grid position u in [0, 1] (u·(gx - 1) = j at node j):
  // v(u) = v_j + (u·(gx - 1) - j)·(v_{j+1} - v_j) = c_j + u·d_j, with d = 0 on the last node, so
  // that a lookup is one FMA on the saturated position (flat beyond the grid)
  for (int j = threadIdx.x; j < gx; j += blockDim.x) {
    const double a = (1.0 - wt) * v0[j] + wt * v1[j];
    const double b = j + 1 < gx ? (1.0 - wt) * v0[j + 1] + wt * v1[j + 1] : a;
    const double d = (double)(gx - 1) * (b - a);
    out[j] = make_float2((float)(a - (double)j * (b - a)), (float)d);
  }
}

void launch_lvrows(const double* lv_v, const int32_t* surf_cell_off, const int32_t* surf_asset,
                   const int2* lv_ti, const double* lv_tw, int n_surf, int T, int gx, float2* rows,
                   cudaStream_t s) {
  if (n_surf <= 0) return;
  lvrows_kernel<<<dim3(n_surf, T), gx < 128 ? 64 : 128, 0, s>>>(lv_v, surf_cell_off, surf_asset, lv_ti,
                                                                lv_tw, T, gx, rows);
  cuda_check(cudaGetLastError(), "lvrows_kernel launch");
}

void launch_calibrate(const CalibJob* jobs_dev, int n_jobs, cudaStream_t s) {
  if (n_jobs <= 0) return;
  calibrate_kernel<<<n_jobs, 128, 0, s>>>(jobs_dev);
  cuda_check(cudaGetLastError(), "calibrate_kernel launch");
}

// ------------------------------------------------------------------ correlation ---------------
// Smallest eigenvalue by cyclic Jacobi (correlation.rs:217-260); `a` holds the n×n matrix and is
// overwritten.
__device__ static double min_eigenvalue_inplace(double* a, int n) {
  if (n == 1) return a[0];
  for (int it = 0; it < 100; ++it) {
    int p = 0, q = 0;
    double mx = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) {
        double v = fabs(a[i * n + j]);
        if (v > mx) { mx = v; p = i; q = j; }
      }
    if (mx < 1.0e-14) break;
    double app = a[p * n + p], aqq = a[q * n + q], apq = a[p * n + q];
    double theta = 0.5 * (aqq - app) / apq;
    double t = copysign(1.0, theta) / (fabs(theta) + sqrt(theta * theta + 1.0));
    double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
    for (int k = 0; k < n; ++k) {
      double akp = a[k * n + p], akq = a[k * n + q];
      a[k * n + p] = cs * akp - sn * akq;
      a[k * n + q] = sn * akp + cs * akq;
    }
    for (int k = 0; k < n; ++k) {
      double apk = a[p * n + k], aqk = a[q * n + k];
      a[p * n + k] = cs * apk - sn * aqk;
      a[q * n + k] = sn * apk + cs * aqk;
    }
  }
  double m = INFINITY;
  for (int i = 0; i < n; ++i) m = fmin(m, a[i * n + i]);
  return m;
}

// L·Lᵀ = C: the matrix as is when its min eigenvalue is >= 1e-10, else PSD-clamped with floor
// 1e-8 (is_positive_semidefinite(-1e-10) and psd_clamp(1e-8), correlation.rs:103-136, 144-148),
// then Cholesky–Banachiewicz (:150-168).  `src` (n×n) is modified, `eig` is n×n scratch.
__device__ static void factor_correlation(double* src, int n, double* l, double* eig) {
  for (int k = 0; k < n * n; ++k) eig[k] = src[k];
  double mn = min_eigenvalue_inplace(eig, n);
  if (!(mn >= 1.0e-10)) {
    double shift = 1.0e-8 - mn;
    for (int k = 0; k < n; ++k) src[k * n + k] += shift;
    for (int k = 0; k < n; ++k) eig[k] = 1.0 / sqrt(src[k * n + k]);
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) src[a * n + b] *= eig[a] * eig[b];
  }
  for (int k = 0; k < n * n; ++k) l[k] = 0.0;
  for (int a = 0; a < n; ++a)
    for (int b = 0; b <= a; ++b) {
      double sum = src[a * n + b];
      for (int k = 0; k < b; ++k) sum -= l[a * n + k] * l[b * n + k];
      if (a == b) {
        l[a * n + b] = sqrt(sum > 0.0 ? sum : 0.0);
      } else {
        double pivot = l[b * n + b];
        l[a * n + b] = pivot > 0.0 ? sum / pivot : 0.0;
      }
    }
}

// One thread per scenario, in place on the scenario's correlation block; the FP32 kernels' copy of
// the factor (rounded once here) when scen32 is given, so their loops convert nothing from FP64.
__global__ void cholesky_kernel(DevScenario* __restrict__ scen, DevScen32* __restrict__ scen32, int n_scen, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_scen) return;
  DevScenario& sc = scen[i];
  double src[RG_NMAX * RG_NMAX], l[RG_NMAX * RG_NMAX], eig[RG_NMAX * RG_NMAX];
  for (int k = 0; k < n * n; ++k) src[k] = sc.L[k];
  factor_correlation(src, n, l, eig);
  for (int k = 0; k < n * n; ++k) sc.L[k] = l[k];
  if (scen32)
    for (int k = 0; k < n * n; ++k) scen32[i].L[k] = (float)l[k];
  sc.status = 0;
}

// One thread for a universe correlation (n <= RG_BOOK_MAX_UNIVERSE); scratch in `work`.
__global__ void cholesky_big_kernel(const double* __restrict__ c, int n, double* __restrict__ l,
                                    double* __restrict__ work) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double* src = work;
  double* eig = work + n * n;
  for (int k = 0; k < n * n; ++k) src[k] = c[k];
  factor_correlation(src, n, l, eig);
}

void launch_cholesky_big(const double* c, int n, double* l, double* work, cudaStream_t s) {
  cholesky_big_kernel<<<1, 32, 0, s>>>(c, n, l, work);
  cuda_check(cudaGetLastError(), "cholesky_big_kernel launch");
}

void launch_cholesky(DevScenario* scen_dev, DevScen32* scen32_dev, int n_scen, int n, cudaStream_t s) {
  cholesky_kernel<<<(n_scen + 63) / 64, 64, 0, s>>>(scen_dev, scen32_dev, n_scen, n);
  cuda_check(cudaGetLastError(), "cholesky_kernel launch");
}

}  // namespace rg
