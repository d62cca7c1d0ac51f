/*
 * riga_oracle.c — CPU oracle (test infrastructure only) for the riga-flow Phoenix hot path.
 *
 * A plain-C FP64 restatement of the reference's CPU algorithm, generalised from two to N assets
 * (QMC dimension of (step, factor) = N·step + factor; the reference's 2·step + factor at N = 2).
 * Each function cites the reference file:line it restates.  Compiled with -ffp-contract=off so
 * that x86-64 and aarch64 hosts give bit-identical results and no FMA contraction differs from
 * the reference's Rust arithmetic.  Only tests, the smoke check and the benchmark's CPU-baseline
 * leg load this library; the product never does.
 */
#include "riga_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NMAX RG_MAX_ASSETS
#define QMC_MAX_DIM 512 /* crates/riga-engine/src/qmc.rs:9 */
#define LV_CLAMP_LO 0.10 /* crates/riga-market/src/lib.rs:30 */
#define LV_CLAMP_HI 3.00 /* crates/riga-market/src/lib.rs:32 */
#define CHUNK_PATHS 4096

static __thread char g_err[512];

static int32_t fail(int32_t status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return status;
}

const char* or_last_error(void) { return g_err; }


/* ============================================================ elementary functions =========== */
/* Two modes for the per-path elementary functions (the Euler step's exp, the local-vol lookup's
 * log of the spot, the probit tails' log).  Default: the platform libm, which is what the
 * reference's Rust f64::exp/ln call — the golden vector is reproduced bit for bit in this mode.
 * Portable: a deterministic exp/log built only from IEEE-754 +, -, *, / and exact power-of-two
 * scaling (Cody–Waite reduction by a split ln 2 and the degree-13 Taylor polynomial; log by the
 * artanh series through s^23), the same published method and coefficients the engine's FP64
 * parity kernel uses on the device, so the two agree bit for bit.  The path-independent values —
 * the Dupire calibration's logarithms and exponentials and the discount factors — are libm's in
 * both modes, as the engine evaluates them on the host with the platform libm.  Compiled with
 * -ffp-contract=off. */
static int g_portable = 0;
void or_set_portable_math(int on) { g_portable = on != 0; }

static double bits_to_double(uint64_t u) { double x; memcpy(&x, &u, sizeof x); return x; }
static uint64_t double_to_bits(double x) { uint64_t u; memcpy(&u, &x, sizeof u); return u; }
static double pow2i(int k) { return bits_to_double((uint64_t)(k + 1023) << 52); }

double or_pexp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return INFINITY;
  if (x < -745.1332191019412) return 0.0;
  const double hi = 0x1.62e42ffp-1, lo = -0x1.718432a1b0e26p-35;
  double k = floor(x * 0x1.71547652b82fep+0 + 0.5);
  double r = (x + -(k * hi)) + -(k * lo);
  static const double c[14] = {0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29, 0x1.ae64567f544e4p-26,
                               0x1.27e4fb7789f5cp-22, 0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16,
                               0x1.a01a01a01a01ap-13, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7,
                               0x1.5555555555555p-5,  0x1.5555555555555p-3,  0.5, 1.0, 1.0};
  double p = c[0];
  for (int i = 1; i < 14; ++i) p = p * r + c[i];
  int ki = (int)k;
  if (ki >= -1022) return ki <= 1023 ? p * pow2i(ki) : (p * pow2i(1023)) * pow2i(ki - 1023);
  return (p * pow2i(ki + 54)) * pow2i(-54);
}

double or_plog(double x) {
  if (x != x) return x;
  if (x < 0.0) return NAN;
  if (x == 0.0) return -INFINITY;
  if (x == INFINITY) return x;
  int e = 0;
  if (x < 0x1p-1022) { x = x * 0x1p54; e = -54; }
  uint64_t b = double_to_bits(x);
  e += (int)((b >> 52) & 0x7ff) - 1023;
  double m = bits_to_double((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m > 0x1.6a09e667f3bcdp+0) { m = m * 0.5; e += 1; }
  double f = m - 1.0, s = f / (2.0 + f), z = s * s;
  static const double c[11] = {0x1.642c8590b2164p-5, 0x1.8618618618618p-5, 0x1.af286bca1af28p-5,
                               0x1.e1e1e1e1e1e1ep-5, 0x1.1111111111111p-4, 0x1.3b13b13b13b14p-4,
                               0x1.745d1745d1746p-4, 0x1.c71c71c71c71cp-4, 0x1.2492492492492p-3,
                               0x1.999999999999ap-3, 0x1.5555555555555p-2};
  double R = c[0];
  for (int i = 1; i < 11; ++i) R = R * z + c[i];
  R = R * z;
  double lm = 2.0 * (s + s * R), ed = (double)e;
  return ed * 0x1.62e42ffp-1 + (lm + ed * -0x1.718432a1b0e26p-35);
}

#define OEXP(x) (g_portable ? or_pexp(x) : exp(x))
#define OLOG(x) (g_portable ? or_plog(x) : log(x))

/* ============================================================ qmc.rs ========================= */

/* Acklam's rational inverse normal CDF, crates/riga-engine/src/qmc.rs:37-91.  The coefficients
 * are Acklam's published ones. */
double or_probit(double p) {
  static const double A[6] = {-3.969683028665376e1, 2.209460984245205e2, -2.759285104469687e2,
                              1.383577518672690e2,  -3.066479806614716e1, 2.506628277459239e0};
  static const double B[5] = {-5.447609879822406e1, 1.615858368580409e2, -1.556989798598866e2,
                              6.680131188771972e1,  -1.328068155288572e1};
  static const double C[6] = {-7.784894002430293e-3, -3.223964580411365e-1, -2.400758277161838e0,
                              -2.549732539343734e0,  4.374664141464968e0,   2.938163982698783e0};
  static const double D[4] = {7.784695709041462e-3, 3.224671290700398e-1, 2.445134137142996e0,
                              3.754408661907416e0};
  if (p <= 0.0) return -INFINITY;
  if (p >= 1.0) return INFINITY;
  const double plow = 0.02425, phigh = 1.0 - plow;
  if (p < plow) {
    double q = sqrt(-2.0 * OLOG(p));
    return (((((C[0] * q + C[1]) * q + C[2]) * q + C[3]) * q + C[4]) * q + C[5]) /
           ((((D[0] * q + D[1]) * q + D[2]) * q + D[3]) * q + 1.0);
  } else if (p <= phigh) {
    double q = p - 0.5, r = q * q;
    return (((((A[0] * r + A[1]) * r + A[2]) * r + A[3]) * r + A[4]) * r + A[5]) * q /
           (((((B[0] * r + B[1]) * r + B[2]) * r + B[3]) * r + B[4]) * r + 1.0);
  } else {
    double q = sqrt(-2.0 * OLOG(1.0 - p));
    return -(((((C[0] * q + C[1]) * q + C[2]) * q + C[3]) * q + C[4]) * q + C[5]) /
           ((((D[0] * q + D[1]) * q + D[2]) * q + D[3]) * q + 1.0);
  }
}

/* van der Corput radical inverse, qmc.rs:24-35 */
double or_radical_inverse(uint64_t index, uint32_t base) {
  double inv = 1.0 / (double)base, factor = inv, result = 0.0;
  while (index > 0) {
    result += factor * (double)(uint32_t)(index % base);
    index /= base;
    factor *= inv;
  }
  return result;
}

/* qmc.rs:12-22 */
int32_t or_first_primes(int32_t count, uint32_t* out) {
  int32_t n = 0;
  for (uint32_t c = 2; n < count; ++c) {
    int prime = 1;
    for (int32_t i = 0; i < n; ++i)
      if (c % out[i] == 0) { prime = 0; break; }
    if (prime) out[n++] = c;
  }
  return n;
}

/* Fisher–Yates digit permutation from an LCG, qmc.rs:128-140 */
void or_halton_permutation(uint32_t base, uint64_t seed, uint32_t* perm) {
  for (uint32_t i = 0; i < base; ++i) perm[i] = i;
  uint64_t state = seed ^ ((uint64_t)base * 0x9E3779B97F4A7C15ULL);
  for (uint32_t i = base - 1; i >= 1; --i) {
    state = state * 6364136223846793005ULL + 1442695040888963407ULL;
    uint64_t j = (state >> 33) % ((uint64_t)i + 1);
    uint32_t t = perm[i];
    perm[i] = perm[j];
    perm[j] = t;
  }
}

/* qmc.rs:143-153 */
static double radical_inverse_scrambled(uint64_t index, uint32_t base, const uint32_t* perm) {
  double inv = 1.0 / (double)base, factor = inv, result = 0.0;
  while (index > 0) {
    result += factor * (double)perm[index % base];
    index /= base;
    factor *= inv;
  }
  return result;
}

/* SplitMix64 finaliser, qmc.rs:310-314 */
uint64_t or_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* The engine's production Halton lane (no counterpart in the reference, whose lane wraps at 512
 * primes): dimension d uses the (d+1)-th prime b, no wrap; digit i of the point (least
 * significant first) goes through x -> (a·x + c) mod b with a in [1, b-1], c in [0, b-1] from a
 * SplitMix64 hash of (seed, d, i); u = R / b^k exactly as the engine forms it. */
double or_halton_hashed_u(uint32_t n, uint32_t b, uint64_t seed, uint64_t dim) {
  const uint64_t key = seed ^ ((dim + 1) * 0xA0761D6478BD642FULL);
  uint64_t R = 0, Bk = 1;
  for (uint32_t i = 0; n; ++i) {
    const uint32_t q = n / b, d = n - q * b;
    const uint64_t h = or_mix64(key ^ ((uint64_t)(i + 1) * 0xE7037ED1A0B428DBULL));
    const uint64_t a = 1u + (((uint64_t)(uint32_t)h * (uint64_t)(b - 1u)) >> 32);
    const uint64_t cc = ((h >> 32) * (uint64_t)b) >> 32;
    R = R * b + (a * d + cc) % b;
    Bk *= b;
    n = q;
  }
  return (double)R / (double)Bk;
}

/* Nested (Owen) scramble keyed on the scrambled prefix, qmc.rs:292-308 */
uint32_t or_owen_scramble(uint32_t x, uint64_t dim, uint64_t seed) {
  uint32_t result = 0, prefix = 0;
  for (int bit = 31; bit >= 0; --bit) {
    uint32_t b = (x >> bit) & 1u;
    uint64_t h = or_mix64(seed ^ (dim * 0x9E3779B97F4A7C15ULL) ^ ((uint64_t)bit * 0xD6E8FEB86659FD93ULL) ^
                          ((uint64_t)prefix * 0xA24BAED4963EE407ULL));
    uint32_t s = b ^ (uint32_t)(h >> 63);
    result |= s << bit;
    prefix = (prefix << 1) | s;
  }
  return result;
}

/* Digital shift (this engine's production scrambler; not in the reference): one 32-bit XOR mask
 * per dimension, the high word of mix64(seed ^ (dim + 1)·0xD1B54A32D192ED03). */
uint32_t or_digital_shift(uint64_t dim, uint64_t seed) {
  return (uint32_t)(or_mix64(seed ^ ((dim + 1) * 0xD1B54A32D192ED03ULL)) >> 32);
}

/* GF(2) arithmetic for the primitivity test, qmc.rs:365-395 */
static int hibit(uint32_t m) { return 31 - __builtin_clz(m); }

static uint32_t gf_mulmod(uint32_t a, uint32_t b, uint32_t mask) {
  int s = hibit(mask);
  uint64_t r = 0, aa = a, bb = b;
  while (bb > 0) {
    if (bb & 1) r ^= aa;
    aa <<= 1;
    bb >>= 1;
  }
  for (int bit = 63; bit >= s; --bit)
    if ((r >> bit) & 1) r ^= (uint64_t)mask << (bit - s);
  return (uint32_t)r;
}

static uint32_t gf_powmod(uint32_t base, uint64_t e, uint32_t mask) {
  uint32_t result = 1, b = base;
  while (e > 0) {
    if (e & 1) result = gf_mulmod(result, b, mask);
    b = gf_mulmod(b, b, mask);
    e >>= 1;
  }
  return result;
}

/* qmc.rs:397-430 */
static int is_primitive(uint32_t mask, int degree) {
  if (degree < 2) return 1;
  uint64_t order = (1ULL << degree) - 1, n = order;
  if (gf_powmod(2, order, mask) != 1) return 0;
  for (uint64_t d = 2; d * d <= n; ++d) {
    if (n % d == 0) {
      if (gf_powmod(2, order / d, mask) == 1) return 0;
      while (n % d == 0) n /= d;
    }
  }
  if (n > 1 && gf_powmod(2, order / n, mask) == 1) return 0;
  return 1;
}

/* Ascending (degree, value) primitive polynomials of degree >= 2, qmc.rs:347-363 */
void or_primitive_polynomials(int64_t count, uint32_t* masks) {
  int64_t got = 0;
  for (int degree = 2; got < count && degree < 31; ++degree) {
    uint32_t lo = 1u << degree, hi = 1u << (degree + 1);
    for (uint32_t mask = lo | 1u; mask < hi && got < count; mask += 2)
      if (is_primitive(mask, degree)) masks[got++] = mask;
  }
}

/* Joe–Kuo recurrence with unit initial values, qmc.rs:316-343 */
void or_direction_numbers(uint32_t mask, uint32_t* v32) {
  int s = hibit(mask);
  uint32_t m[33];
  memset(m, 0, sizeof m);
  for (int i = 1; i <= s; ++i) m[i] = 1;
  for (int k = s + 1; k <= 32; ++k) {
    uint32_t value = ((1u << s) * m[k - s]) ^ m[k - s];
    for (int i = 1; i < s; ++i)
      if ((mask >> (s - i)) & 1u) value ^= (1u << i) * m[k - i];
    m[k] = value;
  }
  for (int k = 0; k < 32; ++k) v32[k] = m[k + 1] << (31 - k);
}

/* Sobol::new, qmc.rs:248-262 */
void or_sobol_table(int64_t dimension, uint32_t* v) {
  for (int k = 0; k < 32; ++k) v[k] = 1u << (31 - k);
  if (dimension <= 1) return;
  uint32_t* masks = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(dimension - 1));
  or_primitive_polynomials(dimension - 1, masks);
  for (int64_t d = 1; d < dimension; ++d) or_direction_numbers(masks[d - 1], v + 32 * d);
  free(masks);
}

/* Sobol::uniform's integer part, qmc.rs:269-279: XOR of v_k over k with an odd count of
 * i in [1, n] of 2-adic valuation k. */
uint32_t or_sobol_int(const uint32_t* v, int64_t dimension, uint64_t n, uint64_t dim) {
  const uint32_t* row = v + 32 * (dim % (uint64_t)dimension);
  uint32_t x = 0;
  for (int k = 0; k < 32; ++k) {
    uint64_t count = (n >> k) - (n >> (k + 1));
    if (count & 1) x ^= row[k];
  }
  return x;
}

/* Depth-first Brownian bridge, qmc.rs:155-191 */
static void bridge_fill(double* path, int64_t lo, int64_t hi, const double* normals, int64_t n,
                        int64_t* index, double dt) {
  if (hi <= lo + 1 || *index >= n) return;
  int64_t mid = (lo + hi) / 2;
  double mean = 0.5 * (path[lo] + path[hi]);
  double variance = ((double)(hi - mid)) * ((double)(mid - lo)) / ((double)(hi - lo)) * dt;
  path[mid] = mean + normals[*index] * sqrt(variance);
  *index += 1;
  bridge_fill(path, lo, mid, normals, n, index, dt);
  bridge_fill(path, mid, hi, normals, n, index, dt);
}

static void bridge_increments_ws(const double* normals, int64_t n, double dt, double* out,
                                 double* path) {
  if (n == 0) return;
  for (int64_t i = 0; i <= n; ++i) path[i] = 0.0;
  path[n] = normals[0] * sqrt((double)n * dt);
  int64_t index = 1;
  bridge_fill(path, 0, n, normals, n, &index, dt);
  for (int64_t t = 0; t < n; ++t) out[t] = path[t + 1] - path[t];
}

void or_bridge_increments(const double* normals, int64_t n, double dt, double* out) {
  double* path = (double*)malloc(sizeof(double) * (size_t)(n + 1));
  bridge_increments_ws(normals, n, dt, out, path);
  free(path);
}

/* ============================================================ correlation.rs ================= */

/* Cyclic Jacobi eigenvalues, crates/riga-market/src/correlation.rs:217-260 */
static void jacobi_eigenvalues(double* a, int n, double* eig) {
  if (n == 1) { eig[0] = a[0]; return; }
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
    double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
    for (int k = 0; k < n; ++k) {
      double akp = a[k * n + p], akq = a[k * n + q];
      a[k * n + p] = c * akp - s * akq;
      a[k * n + q] = s * akp + c * akq;
    }
    for (int k = 0; k < n; ++k) {
      double apk = a[p * n + k], aqk = a[q * n + k];
      a[p * n + k] = c * apk - s * aqk;
      a[q * n + k] = s * apk + c * aqk;
    }
  }
  for (int i = 0; i < n; ++i) eig[i] = a[i * n + i];
}

/* correlation.rs:95-101 */
double or_min_eigenvalue(const double* c, int32_t n) {
  double a[NMAX * NMAX * 16], e[NMAX * 4];
  if (n > NMAX * 4) return NAN;
  memcpy(a, c, sizeof(double) * (size_t)(n * n));
  jacobi_eigenvalues(a, n, e);
  double m = INFINITY;
  for (int i = 0; i < n; ++i) m = fmin(m, e[i]);
  return m;
}

/* Diagonal loading + unit-diagonal rescale, correlation.rs:108-136 */
void or_psd_clamp(const double* c, int32_t n, double floor_, double* out) {
  double mn = or_min_eigenvalue(c, n);
  memcpy(out, c, sizeof(double) * (size_t)(n * n));
  if (mn >= floor_) return;
  double shift = floor_ - mn, inv[NMAX * 4];
  for (int i = 0; i < n; ++i) out[i * n + i] += shift;
  for (int i = 0; i < n; ++i) inv[i] = 1.0 / sqrt(out[i * n + i]);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) out[i * n + j] *= inv[i] * inv[j];
}

/* CorrelationMatrix::validate (correlation.rs:74-93) + cholesky (correlation.rs:138-168) */
int32_t or_cholesky(const double* c, int32_t n, double* l) {
  if (n <= 0 || n > NMAX * 4) return fail(RG_ERR_INVALID_MARKET, "correlation matrix must have at least one factor");
  for (int i = 0; i < n; ++i) {
    if (fabs(c[i * n + i] - 1.0) > 1.0e-9)
      return fail(RG_ERR_INVALID_MARKET, "correlation diagonal [%d] must be exactly one", i);
    for (int j = 0; j < n; ++j) {
      double v = c[i * n + j];
      if (!isfinite(v)) return fail(RG_ERR_INVALID_MARKET, "correlation entries must be finite");
      if (fabs(v) > 1.0 + 1.0e-9)
        return fail(RG_ERR_INVALID_MARKET, "correlation [%d,%d]=%g is outside [-1, 1]", i, j, v);
      if (fabs(v - c[j * n + i]) > 1.0e-9)
        return fail(RG_ERR_INVALID_MARKET, "correlation [%d,%d] is not symmetric", i, j);
    }
  }
  double src[NMAX * NMAX * 16];
  /* is_positive_semidefinite(-1e-10) is min_eigenvalue >= 1e-10 (correlation.rs:103-106,144) */
  if (or_min_eigenvalue(c, n) >= 1.0e-10)
    memcpy(src, c, sizeof(double) * (size_t)(n * n));
  else
    or_psd_clamp(c, n, 1.0e-8, src);
  for (int i = 0; i < n * n; ++i) l[i] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double sum = src[i * n + j];
      for (int k = 0; k < j; ++k) sum -= l[i * n + k] * l[j * n + k];
      if (i == j) {
        l[i * n + j] = sqrt(sum > 0.0 ? sum : 0.0);
      } else {
        double pivot = l[j * n + j];
        l[i * n + j] = pivot > 0.0 ? sum / pivot : 0.0;
      }
    }
  return RG_OK;
}

/* ============================================================ riga-market/src/lib.rs ========= */

/* Natural-spline second derivatives (Thomas solve), crates/riga-market/src/lib.rs:125-176 */
static void natural_second_derivatives(const double* x, const double* y, int n, double* y2) {
  for (int i = 0; i < n; ++i) y2[i] = 0.0;
  if (n < 3) return;
  double *h = (double*)calloc((size_t)n, sizeof(double)), *a = (double*)calloc((size_t)n, sizeof(double)),
         *b = (double*)calloc((size_t)n, sizeof(double)), *c = (double*)calloc((size_t)n, sizeof(double)),
         *d = (double*)calloc((size_t)n, sizeof(double)), *cp = (double*)calloc((size_t)n, sizeof(double)),
         *dp = (double*)calloc((size_t)n, sizeof(double));
  int bad = 0;
  for (int i = 0; i < n - 1; ++i) {
    h[i] = x[i + 1] - x[i];
    if (h[i] <= 0.0) bad = 1;
  }
  for (int i = 0; i < n; ++i)
    if (!isfinite(y[i])) bad = 1;
  if (!bad) {
    b[0] = 1.0;
    b[n - 1] = 1.0;
    for (int i = 1; i < n - 1; ++i) b[i] = 2.0 * (h[i - 1] + h[i]);
    for (int i = 1; i < n; ++i) a[i] = i < n - 1 ? h[i] : 0.0;
    for (int i = 0; i < n - 1; ++i) c[i] = i + 1 < n - 1 ? h[i + 1] : 0.0;
    for (int i = 1; i < n - 1; ++i) d[i] = 6.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1]);
    cp[0] = c[0] / b[0];
    dp[0] = d[0] / b[0];
    for (int i = 1; i < n; ++i) {
      double m = b[i] - a[i] * cp[i - 1];
      if (fabs(m) < 1e-300) m = 1e-300;
      cp[i] = c[i] / m;
      dp[i] = (d[i] - a[i] * dp[i - 1]) / m;
    }
    y2[n - 1] = dp[n - 1];
    for (int i = n - 2; i >= 0; --i) y2[i] = dp[i] - cp[i] * y2[i + 1];
  }
  free(h); free(a); free(b); free(c); free(d); free(cp); free(dp);
}

/* Spline value and derivatives, crates/riga-market/src/lib.rs:178-203 (term order kept, including
 * its placement of y2[seg] and y2[seg+1]). */
static void spline_eval1(double p, const double* x, const double* y, const double* y2, int n,
                         double* f, double* f1, double* f2) {
  int seg = 0;
  while (seg + 1 < n - 1 && p > x[seg + 1]) seg += 1;
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

static int32_t validate_grid(const rg_implied_vol_grid* g) {
  if (!g || g->n_maturities <= 0 || g->n_strikes <= 0 || !g->maturities_years || !g->strikes || !g->vols)
    return fail(RG_ERR_INVALID_LOCAL_VOL, "implied vol grid has an empty axis");
  for (int i = 0; i + 1 < g->n_maturities; ++i)
    if (!(g->maturities_years[i] < g->maturities_years[i + 1]))
      return fail(RG_ERR_INVALID_LOCAL_VOL, "implied vol maturities must be strictly increasing");
  for (int i = 0; i + 1 < g->n_strikes; ++i)
    if (!(g->strikes[i] < g->strikes[i + 1]))
      return fail(RG_ERR_INVALID_LOCAL_VOL, "implied vol strikes must be strictly increasing");
  return RG_OK;
}

/* DupireLocalVol::calibrate, crates/riga-market/src/lib.rs:205-299 (gx = GRID_X = 96 there). */
int32_t or_lv_calibrate(const rg_implied_vol_grid* grid, double spot, double rate, int32_t gx,
                        or_lv_surface* out) {
  memset(out, 0, sizeof *out);
  int32_t st = validate_grid(grid);
  if (st) return st;
  if (!isfinite(spot) || spot <= 0.0)
    return fail(RG_ERR_INVALID_LOCAL_VOL, "local-vol calibration needs a positive finite spot");
  if (gx < 2) return fail(RG_ERR_INVALID_LOCAL_VOL, "local-vol grid needs at least two points");
  int nt = grid->n_maturities, nk = grid->n_strikes;
  const double* K = grid->strikes;
  double s_min = K[0] * 0.55, s_max = K[nk - 1] * 1.05;
  /* the calibration's logarithms and exponentials are libm's in both math modes: the engine
     evaluates them on the host with the platform libm too */
  double log_lo = log(s_min > 1e-6 ? s_min : 1e-6), log_hi = log(s_max > 1e-6 ? s_max : 1e-6);
  out->n_t = nt;
  out->gx = gx;
  out->t_axis = (double*)malloc(sizeof(double) * (size_t)nt);
  out->log_s = (double*)malloc(sizeof(double) * (size_t)gx);
  out->v = (double*)malloc(sizeof(double) * (size_t)(nt * gx));
  memcpy(out->t_axis, grid->maturities_years, sizeof(double) * (size_t)nt);
  double* s_axis = (double*)malloc(sizeof(double) * (size_t)gx);
  for (int i = 0; i < gx; ++i) {
    out->log_s[i] = log_lo + (log_hi - log_lo) * (double)i / (double)(gx - 1);
    s_axis[i] = exp(out->log_s[i]);
  }
  size_t cells = (size_t)nt * (size_t)gx;
  double *w = (double*)malloc(sizeof(double) * cells), *wx = (double*)malloc(sizeof(double) * cells),
         *wxx = (double*)malloc(sizeof(double) * cells), *xa = (double*)malloc(sizeof(double) * cells);
  double *xj = (double*)malloc(sizeof(double) * (size_t)nk), *y2 = (double*)malloc(sizeof(double) * (size_t)nk);
  for (int k = 0; k < nt; ++k) {
    double tk = grid->maturities_years[k];
    double forward = spot * exp(rate * tk);
    for (int j = 0; j < nk; ++j) xj[j] = log(K[j] / forward);
    const double* y = grid->vols + (size_t)k * nk;
    natural_second_derivatives(xj, y, nk, y2);
    double x_lo = xj[0], x_hi = xj[nk - 1];
    for (int i = 0; i < gx; ++i) {
      double xd = log(s_axis[i] / forward);
      xd = xd < x_lo ? x_lo : (xd > x_hi ? x_hi : xd);
      double sg, s1, s2;
      if (nk >= 2) {
        spline_eval1(xd, xj, y, y2, nk, &sg, &s1, &s2);
      } else {
        sg = y[0]; s1 = 0.0; s2 = 0.0; /* one strike: the reference indexes past the end */
      }
      size_t c = (size_t)k * gx + i;
      w[c] = sg * sg * tk;
      wx[c] = 2.0 * sg * tk * s1;
      wxx[c] = 2.0 * tk * (s1 * s1 + sg * s2);
      xa[c] = xd;
    }
  }
  const double* T = grid->maturities_years;
  for (int k = 0; k < nt; ++k)
    for (int i = 0; i < gx; ++i) {
      double dw;
      if (nt == 1) {
        dw = w[i] / (T[0] > 1e-9 ? T[0] : 1e-9);
      } else if (k == 0) {
        double sp = T[1] - T[0];
        dw = (w[(size_t)gx + i] - w[i]) / (sp > 1e-9 ? sp : 1e-9);
      } else if (k == nt - 1) {
        double sp = T[nt - 1] - T[nt - 2];
        dw = (w[(size_t)(nt - 1) * gx + i] - w[(size_t)(nt - 2) * gx + i]) / (sp > 1e-9 ? sp : 1e-9);
      } else {
        double sp = T[k + 1] - T[k - 1];
        dw = (w[(size_t)(k + 1) * gx + i] - w[(size_t)(k - 1) * gx + i]) / (sp > 1e-9 ? sp : 1e-9);
      }
      size_t c = (size_t)k * gx + i;
      double ww = w[c] > 1e-12 ? w[c] : 1e-12;
      double denom = 1.0 - (xa[c] / ww) * wx[c] + 0.25 * (-0.25 - 1.0 / ww) * wx[c] * wx[c] + 0.5 * wxx[c];
      double lv2 = (isfinite(denom) && fabs(denom) > 1e-12) ? dw / denom : LV_CLAMP_LO * LV_CLAMP_LO;
      double lo2 = LV_CLAMP_LO * LV_CLAMP_LO, hi2 = LV_CLAMP_HI * LV_CLAMP_HI;
      lv2 = lv2 < lo2 ? lo2 : (lv2 > hi2 ? hi2 : lv2);
      out->v[c] = sqrt(lv2);
    }
  free(s_axis); free(w); free(wx); free(wxx); free(xa); free(xj); free(y2);
  return RG_OK;
}

void or_lv_free(or_lv_surface* s) {
  free(s->t_axis); free(s->log_s); free(s->v);
  memset(s, 0, sizeof *s);
}

/* DupireLocalVol::sigma, crates/riga-market/src/lib.rs:301-343 */
double or_lv_sigma(const or_lv_surface* s, double t, double spot) {
  double x = OLOG(spot > 1e-12 ? spot : 1e-12);
  int n = s->gx, lo, hi;
  if (x <= s->log_s[0]) { lo = 0; hi = 0; }
  else if (x >= s->log_s[n - 1]) { lo = n - 1; hi = n - 1; }
  else {
    int j = 0;
    while (j + 1 < n && x > s->log_s[j + 1]) j += 1;
    lo = j; hi = j + 1;
  }
  double wx = hi == lo ? 0.0 : (x - s->log_s[lo]) / (s->log_s[hi] - s->log_s[lo]);
  int i, i1;
  double wt;
  if (s->n_t == 1) { i = 0; i1 = 0; wt = 0.0; }
  else {
    double t0 = s->t_axis[0], tn = s->t_axis[s->n_t - 1];
    double tc = t < t0 ? t0 : (t > tn ? tn : t);
    int ii = 0;
    while (ii + 1 < s->n_t - 1 && tc > s->t_axis[ii + 1]) ii += 1;
    double span = s->t_axis[ii + 1] - s->t_axis[ii];
    wt = span > 0.0 ? (tc - s->t_axis[ii]) / span : 0.0;
    i = ii; i1 = ii + 1;
  }
  const double* v = s->v;
  double v0 = (1.0 - wx) * v[i * n + lo] + wx * v[i * n + hi];
  double v1 = (1.0 - wx) * v[i1 * n + lo] + wx * v[i1 * n + hi];
  return (1.0 - wt) * v0 + wt * v1;
}

/* ============================================================ lib.rs validate ================ */

/* crates/riga-engine/src/lib.rs:209-321, generalised to 1..RG_MAX_ASSETS assets. */
int32_t or_validate(const rg_price_request* r) {
  const rg_phoenix_trade* t = &r->trade;
  const rg_market_snapshot* m = &r->market;
  const rg_simulation_config* c = &r->config;
  if (!r->as_of || r->as_of[0] == 0) return fail(RG_ERR_MISSING_AS_OF, "as_of is required");
  if (!m->as_of || strcmp(r->as_of, m->as_of) != 0)
    return fail(RG_ERR_AS_OF_MISMATCH, "request as_of must match the market snapshot as_of");
  if (c->paths == 0 || c->path_block_size == 0)
    return fail(RG_ERR_INVALID_PATHS, "paths and path_block_size must be positive");
  if (t->steps <= 0 || !isfinite(t->maturity_years) || t->maturity_years <= 0.0)
    return fail(RG_ERR_INVALID_SCHEDULE, "steps and maturity_years must be positive and finite");
  int n = m->n_assets;
  if (n < 1 || n > NMAX || t->n_assets != n || !m->spots || !m->vols || !m->dividend_yields ||
      !m->correlation || !t->initial_spots)
    return fail(RG_ERR_INVALID_MARKET_SHAPE, "the engine requires 1..%d assets with aligned trade and market arrays", NMAX);
  for (int f = 0; f < n; ++f) {
    if (!isfinite(m->spots[f])) return fail(RG_ERR_INVALID_MARKET, "spot[%d] must be finite", f);
    if (!isfinite(m->vols[f])) return fail(RG_ERR_INVALID_MARKET, "vol[%d] must be finite", f);
  }
  if (!isfinite(m->risk_free_rate)) return fail(RG_ERR_INVALID_MARKET, "risk_free_rate must be finite");
  for (int f = 0; f < n; ++f) {
    if (!isfinite(m->dividend_yields[f])) return fail(RG_ERR_INVALID_MARKET, "dividend_yield[%d] must be finite", f);
    if (!isfinite(t->initial_spots[f])) return fail(RG_ERR_INVALID_MARKET, "initial_spot[%d] must be finite", f);
  }
  for (int i = 0; i < n * n; ++i)
    if (!isfinite(m->correlation[i])) return fail(RG_ERR_INVALID_MARKET, "rho must be finite");
  if (!isfinite(t->strike)) return fail(RG_ERR_INVALID_MARKET, "strike must be finite");
  if (!isfinite(t->knock_in_barrier)) return fail(RG_ERR_INVALID_MARKET, "KI barrier must be finite");
  int bad = 0;
  for (int f = 0; f < n; ++f)
    if (m->spots[f] <= 0.0 || t->initial_spots[f] <= 0.0 || m->vols[f] < 0.0) bad = 1;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double v = m->correlation[i * n + j];
      if (i == j) { if (fabs(v - 1.0) > 1.0e-12) bad = 1; }
      else if (fabs(v) > 1.0 || fabs(v - m->correlation[j * n + i]) > 1.0e-12) bad = 1;
    }
  if (bad)
    return fail(RG_ERR_INVALID_MARKET, "spots must be positive, vols non-negative, and correlation in [-1,1]");
  if (t->has_knock_out_barrier && (!isfinite(t->knock_out_barrier) || t->knock_out_barrier <= 0.0))
    return fail(RG_ERR_INVALID_TRADE, "knock_out_barrier must be finite and positive when present");
  if (t->has_coupon_barrier && (!isfinite(t->coupon_barrier) || t->coupon_barrier <= 0.0))
    return fail(RG_ERR_INVALID_TRADE, "coupon_barrier must be finite and positive when present");
  if (t->has_coupon_rate && (!isfinite(t->coupon_rate) || t->coupon_rate < 0.0))
    return fail(RG_ERR_INVALID_TRADE, "coupon_rate must be finite and non-negative when present");
  if (t->strike <= 0.0 || t->knock_in_barrier <= 0.0)
    return fail(RG_ERR_INVALID_TRADE, "strike must be positive and barriers finite");
  if (r->n_local_vol != 0 && r->n_local_vol != n)
    return fail(RG_ERR_INVALID_LOCAL_VOL, "local_vol.grids must be aligned with market.spots");
  if (r->n_local_vol != 0 && !r->local_vol)
    return fail(RG_ERR_INVALID_LOCAL_VOL, "local_vol.grids must be aligned with market.spots");
  if (c->variance_reduction < RG_VR_NONE || c->variance_reduction > RG_VR_SOBOL)
    return fail(RG_ERR_INVALID_ARGUMENT, "unknown variance_reduction %d", c->variance_reduction);
  return RG_OK;
}

/* ============================================================ MC lane normals ================ */
/* The reference's pseudo-random lane draws `ChaCha8Rng::seed_from_u64(seed)` (rand_chacha 0.9.0,
 * rand_core 0.9.5) and `rand_distr::StandardNormal` (rand_distr 0.5.1), note.rs:58,123-127.
 * Those crates are not part of the reference checkout; this restates their published algorithms:
 *  - seed_from_u64: the 32-byte seed is eight little-endian PCG32 outputs of the seed state
 *    (MUL 6364136223846793005, INC 11634580027462260723, XSH-RR output);
 *  - ChaCha with 8 rounds, 64-bit block counter in words 12-13 from 0, stream 0 in words 14-15;
 *    next_u64 = low word | high word << 32 of consecutive output words;
 *  - Doornik's ZIGNOR ziggurat with 256 layers (R = 3.6541528853610088, V = 0.00492867323399);
 *    the layer tables are regenerated here from that recurrence and rounded to the 18 decimal
 *    places the crate's table literals carry. */
typedef struct chacha8 {
  uint32_t key[8];
  uint64_t counter;
  uint32_t buf[16];
  int idx;
} chacha8;

static uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

#define QR(a, b, c, d)                                                                    \
  x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 16); x[c] += x[d]; x[b] ^= x[c];        \
  x[b] = rotl32(x[b], 12); x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 8); x[c] += x[d]; \
  x[b] ^= x[c]; x[b] = rotl32(x[b], 7);

static void chacha8_block(chacha8* g) {
  uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
  for (int i = 0; i < 8; ++i) s[4 + i] = g->key[i];
  s[12] = (uint32_t)g->counter;
  s[13] = (uint32_t)(g->counter >> 32);
  s[14] = 0;
  s[15] = 0;
  uint32_t x[16];
  memcpy(x, s, sizeof x);
  for (int r = 0; r < 4; ++r) {
    QR(0, 4, 8, 12) QR(1, 5, 9, 13) QR(2, 6, 10, 14) QR(3, 7, 11, 15)
    QR(0, 5, 10, 15) QR(1, 6, 11, 12) QR(2, 7, 8, 13) QR(3, 4, 9, 14)
  }
  for (int i = 0; i < 16; ++i) g->buf[i] = x[i] + s[i];
  g->counter += 1;
  g->idx = 0;
}

static void chacha8_seed_u64(chacha8* g, uint64_t state) {
  for (int i = 0; i < 8; ++i) {
    state = state * 6364136223846793005ULL + 11634580027462260723ULL;
    uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
    uint32_t rot = (uint32_t)(state >> 59);
    g->key[i] = (xorshifted >> rot) | (xorshifted << ((32 - rot) & 31));
  }
  g->counter = 0;
  g->idx = 16;
}

static uint64_t chacha8_u64(chacha8* g) {
  if (g->idx >= 16) chacha8_block(g);
  uint64_t lo = g->buf[g->idx], hi = g->buf[g->idx + 1];
  g->idx += 2;
  return lo | (hi << 32);
}

#define ZIG_NORM_R 3.6541528853610088
static double zig_x[257], zig_f[257];
static pthread_once_t zig_once = PTHREAD_ONCE_INIT;

static double round18(double v) {
  char b[64];
  snprintf(b, sizeof b, "%.18f", v);
  return strtod(b, NULL);
}

static void zig_init(void) {
  const double r = ZIG_NORM_R, v = 0.00492867323399;
  double x[257];
  x[0] = v / exp(-r * r / 2.0);
  x[1] = r;
  for (int i = 2; i < 256; ++i) {
    double last = x[i - 1];
    x[i] = sqrt(-2.0 * log(v / last + exp(-last * last / 2.0)));
  }
  x[256] = 0.0;
  for (int i = 0; i < 257; ++i) {
    zig_x[i] = round18(x[i]);
    zig_f[i] = round18(exp(-x[i] * x[i] / 2.0));
  }
}

static double bits_to_float_exp(uint64_t frac52, int e) {
  uint64_t b = frac52 | ((uint64_t)(1023 + e) << 52);
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
}

static double open01(chacha8* g) {
  return bits_to_float_exp(chacha8_u64(g) >> 12, 0) - (1.0 - 2.220446049250313e-16 / 2.0);
}

static double std_uniform(chacha8* g) {
  return (double)(chacha8_u64(g) >> 11) * (1.0 / 9007199254740992.0);
}

static double zig_normal(chacha8* g) {
  for (;;) {
    uint64_t bits = chacha8_u64(g);
    int i = (int)(bits & 0xff);
    double u = bits_to_float_exp(bits >> 12, 1) - 3.0;
    double x = u * zig_x[i];
    if (fabs(x) < zig_x[i + 1]) return x;
    if (i == 0) {
      double xx = 1.0, y = 0.0;
      while (-2.0 * y < xx * xx) {
        double x_ = open01(g), y_ = open01(g);
        xx = log(x_) / ZIG_NORM_R;
        y = log(y_);
      }
      return u < 0.0 ? xx - ZIG_NORM_R : ZIG_NORM_R - xx;
    }
    if (zig_f[i + 1] + (zig_f[i] - zig_f[i + 1]) * std_uniform(g) < exp(-x * x / 2.0)) return x;
  }
}

/* First `count` StandardNormal draws of ChaCha8Rng::seed_from_u64(seed) (test hook). */
void or_chacha8_normals(uint64_t seed, uint64_t count, double* out) {
  pthread_once(&zig_once, zig_init);
  chacha8 g;
  chacha8_seed_u64(&g, seed);
  for (uint64_t i = 0; i < count; ++i) out[i] = zig_normal(&g);
}

void or_chacha8_u64(uint64_t seed, uint64_t count, uint64_t* out) {
  chacha8 g;
  chacha8_seed_u64(&g, seed);
  for (uint64_t i = 0; i < count; ++i) out[i] = chacha8_u64(&g);
}

/* ============================================================ note.rs pricer ================= */

typedef struct model {
  int n;
  int64_t steps, periods, call_start;
  double dt, rate, maturity;
  double spots[NMAX], init[NMAX], vols[NMAX], q[NMAX];
  double L[RG_BOOK_MAX_UNIVERSE * RG_BOOK_MAX_UNIVERSE]; /* n × n, row-major */
  double call_barrier, coupon_barrier, coupon_rate, strike, ki;
  int fixed_first, memory, trace;
  int has_lv;
  or_lv_surface lv[NMAX];
  int vr, scrambler;
  uint64_t seed, first_path;
  uint32_t* sob_v;
  int64_t sob_dim;
  uint32_t* hal_bases;
  uint32_t** hal_perm;
  int32_t hal_dim;
  int hal_hash; /* the engine's production Halton lane (full dimensions, hashed affine digits) */
} model;

static void model_free(model* m) {
  for (int f = 0; f < NMAX; ++f) or_lv_free(&m->lv[f]);
  free(m->sob_v);
  if (m->hal_perm)
    for (int i = 0; i < m->hal_dim; ++i) free(m->hal_perm[i]);
  free(m->hal_perm);
  free(m->hal_bases);
  memset(m, 0, sizeof *m);
}

/* QMC tables of a model with `need` = N·T normals per path (Ladder set-up, note.rs:58-63,
 * qmc.rs:93-117, 247-262). */
static void qmc_init(model* m, const rg_simulation_config* c, int64_t need) {
  m->vr = c->variance_reduction;
  m->seed = c->seed;
  m->first_path = c->first_path;
  m->scrambler = c->scrambler;
  if (m->vr == RG_VR_SOBOL) {
    int64_t d = (int64_t)c->qmc_dimension;
    if (c->dim_mode == RG_DIM_FULL) {
      if (d < need) d = need;
    } else {
      if (d < 1) d = 1;
      if (d > QMC_MAX_DIM) d = QMC_MAX_DIM;
    }
    m->sob_dim = d;
    m->sob_v = (uint32_t*)malloc(sizeof(uint32_t) * 32 * (size_t)d);
    or_sobol_table(d, m->sob_v);
  } else if (m->vr == RG_VR_HALTON && c->dim_mode == RG_DIM_FULL) {
    int64_t d = (int64_t)c->qmc_dimension;
    if (d < need) d = need;
    m->hal_dim = (int32_t)d;
    m->hal_hash = 1;
    m->hal_bases = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)d);
    or_first_primes((int32_t)d, m->hal_bases);
  } else if (m->vr == RG_VR_HALTON) {
    int64_t d = (int64_t)c->qmc_dimension;
    if (d < 1) d = 1;
    if (d > QMC_MAX_DIM) d = QMC_MAX_DIM;
    m->hal_dim = (int32_t)d;
    m->hal_bases = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)d);
    or_first_primes((int32_t)d, m->hal_bases);
    m->hal_perm = (uint32_t**)calloc((size_t)d, sizeof(uint32_t*));
    for (int i = 0; i < d; ++i) {
      m->hal_perm[i] = (uint32_t*)malloc(sizeof(uint32_t) * m->hal_bases[i]);
      or_halton_permutation(m->hal_bases[i], m->seed, m->hal_perm[i]);
    }
  }
}

/* price_full_phoenix set-up, note.rs:38-63 and build_local_vol, lib.rs:326-343.
 * `vol_shift` is an optional per-asset parallel implied-vol shift (riga-risk lib.rs:260-279). */
static int32_t model_init(model* m, const rg_price_request* r, const rg_market_snapshot* mk,
                          const double* vol_shift) {
  memset(m, 0, sizeof *m);
  const rg_phoenix_trade* t = &r->trade;
  int n = m->n = mk->n_assets;
  m->steps = t->steps;
  m->periods = t->has_coupon_periods ? t->coupon_periods : 9;
  if (m->periods < 1) m->periods = 1;
  m->call_start = t->has_call_start_step ? t->call_start_step : 0;
  m->dt = t->maturity_years / (double)t->steps;
  m->rate = mk->risk_free_rate;
  m->maturity = t->maturity_years;
  for (int f = 0; f < n; ++f) {
    m->spots[f] = mk->spots[f];
    m->init[f] = t->initial_spots[f];
    m->vols[f] = mk->vols[f];
    m->q[f] = mk->dividend_yields[f];
  }
  m->call_barrier = t->has_knock_out_barrier ? t->knock_out_barrier : INFINITY;
  m->coupon_barrier = t->has_coupon_barrier ? t->coupon_barrier : INFINITY;
  m->coupon_rate = t->has_coupon_rate ? t->coupon_rate : 0.0;
  m->strike = t->strike;
  m->ki = t->knock_in_barrier;
  m->fixed_first = t->fixed_first_coupon != 0;
  m->memory = t->memory_coupon != 0;
  m->trace = r->config.trace_level != RG_TRACE_OFF;
  int32_t st;
  if (r->n_local_vol) {
    m->has_lv = 1;
    int gx = r->config.lv_grid_x > 0 ? r->config.lv_grid_x : 96;
    for (int f = 0; f < n; ++f) {
      rg_implied_vol_grid g = r->local_vol[f];
      double* shifted = NULL;
      if (vol_shift && vol_shift[f] != 0.0 && g.vols) {
        size_t cnt = (size_t)g.n_maturities * (size_t)g.n_strikes;
        shifted = (double*)malloc(sizeof(double) * cnt);
        for (size_t i = 0; i < cnt; ++i) shifted[i] = g.vols[i] + vol_shift[f];
        g.vols = shifted;
      }
      st = or_lv_calibrate(&g, mk->spots[f], mk->risk_free_rate, gx, &m->lv[f]);
      free(shifted);
      if (st) { model_free(m); return st; }
    }
  }
  st = or_cholesky(mk->correlation, n, m->L);
  if (st) { model_free(m); return st; }
  qmc_init(m, &r->config, (int64_t)n * m->steps);
  return RG_OK;
}

/* Ladder::normal for the QMC lanes, qmc.rs:119-125, 284-289 */
static double ladder_normal(const model* m, uint64_t point, uint64_t dim) {
  double u;
  if (m->vr == RG_VR_SOBOL) {
    uint32_t x = or_sobol_int(m->sob_v, m->sob_dim, point + 1, dim);
    x = m->scrambler == RG_SCRAMBLE_DIGITAL_SHIFT ? x ^ or_digital_shift(dim, m->seed)
                                                  : or_owen_scramble(x, dim, m->seed);
    u = ((double)x + 0.5) / 4294967296.0;
  } else if (m->hal_hash) {
    u = or_halton_hashed_u((uint32_t)(point + 1), m->hal_bases[dim], m->seed, dim);
  } else {
    uint64_t idx = dim % (uint64_t)m->hal_dim;
    u = radical_inverse_scrambled(point + 1, m->hal_bases[idx], m->hal_perm[idx]);
  }
  u = u < 1.0e-12 ? 1.0e-12 : (u > 1.0 - 1.0e-12 ? 1.0 - 1.0e-12 : u);
  return or_probit(u);
}

typedef struct path_out {
  double worst_final, redemption_time, put, coupon_pv, memory_pv, funding, pv;
  int ko, ko_step, hit_ki, put_eligible, received, qualified, paid;
} path_out;

typedef struct workspace {
  double* normals; /* [n][T] */
  double* incr;    /* [n][T] */
  double* path;    /* [T+1] */
} workspace;

static void ws_alloc(workspace* w, int n, int64_t T) {
  w->normals = (double*)malloc(sizeof(double) * (size_t)n * (size_t)T);
  w->incr = (double*)malloc(sizeof(double) * (size_t)n * (size_t)T);
  w->path = (double*)malloc(sizeof(double) * (size_t)(T + 1));
}
static void ws_free(workspace* w) { free(w->normals); free(w->incr); free(w->path); }

/* Cholesky::apply_into, correlation.rs:195-206 */
static void chol_apply(const double* L, int n, const double* z, double* y) {
  for (int i = 0; i < n; ++i) {
    double acc = 0.0;
    for (int j = 0; j <= i; ++j) acc += L[i * n + j] * z[j];
    y[i] = acc;
  }
}

/* Normals → correlation → bridge of one path (note.rs:83-127): ws->incr[f][step] = ΔW/√dt. */
static void path_increments(const model* m, uint64_t path_id, workspace* ws, chacha8* mc) {
  const int n = m->n;
  const int64_t T = m->steps;
  const double dt = m->dt;
  double z[RG_BOOK_MAX_UNIVERSE], y[RG_BOOK_MAX_UNIVERSE];
  if (m->vr == RG_VR_NONE) {
    /* pseudo-random lane: n draws per step then L·z, note.rs:123-127 */
    for (int64_t s = 0; s < T; ++s) {
      for (int f = 0; f < n; ++f) z[f] = zig_normal(mc);
      chol_apply(m->L, n, z, y);
      for (int f = 0; f < n; ++f) ws->incr[(size_t)f * T + s] = y[f];
    }
  } else {
    /* per-path QMC normals, Cholesky, bridge, note.rs:83-106 */
    for (int64_t s = 0; s < T; ++s) {
      for (int f = 0; f < n; ++f) z[f] = ladder_normal(m, m->first_path + path_id, (uint64_t)(s * n + f));
      chol_apply(m->L, n, z, y);
      for (int f = 0; f < n; ++f) ws->normals[(size_t)f * T + s] = y[f];
    }
    double inv_sqrt_dt = 1.0 / sqrt(dt);
    for (int f = 0; f < n; ++f) {
      bridge_increments_ws(ws->normals + (size_t)f * T, T, dt, ws->incr + (size_t)f * T, ws->path);
      for (int64_t s = 0; s < T; ++s) ws->incr[(size_t)f * T + s] *= inv_sqrt_dt;
    }
  }
}

/* The Euler step and the Phoenix scan of one path (note.rs:129-259) over increment rows
 * incr[f][0..steps-1].  When `cube` is non-null it receives the spots after every step as
 * f32, cube[step * n + f] (explain.rs:183-193 state; pathcube.rs:19-35 layout). */
static void scan_path_cube(const model* m, const double* const* incr, path_out* o, float* cube) {
  const int n = m->n;
  const int64_t T = m->steps;
  const double dt = m->dt;
  double spots[NMAX];
  for (int f = 0; f < n; ++f) spots[f] = m->spots[f];
  int ko = 0, received = 0;
  double redemption_time = m->maturity, accrual = 0.0, unpaid = 0.0, coupon_pv = 0.0, memory_pv = 0.0;
  int64_t current_period = 0;
  double final_worst = 1.0;
  memset(o, 0, sizeof *o);
  o->ko_step = -1;
  for (int64_t step = 0; step < T; ++step) {
    int active = !ko;
    double time = (double)(step + 1) * dt;
    for (int f = 0; f < n; ++f) {
      double vol = m->has_lv ? or_lv_sigma(&m->lv[f], (double)step * dt, spots[f]) : m->vols[f];
      double drift = (m->rate - m->q[f] - 0.5 * vol * vol) * dt;
      spots[f] *= OEXP(drift + vol * sqrt(dt) * incr[f][step]);
    }
    if (cube)
      for (int f = 0; f < n; ++f) cube[step * n + f] = (float)spots[f];
    double worst = spots[0] / m->init[0];
    for (int f = 1; f < n; ++f) worst = fmin(worst, spots[f] / m->init[f]);
    final_worst = worst;
    if (!active) continue;
    int64_t period = (step * m->periods) / T;
    if (period > m->periods - 1) period = m->periods - 1;
    if (period != current_period) { current_period = period; accrual = 0.0; }
    if (period == 0 && m->fixed_first) {
    } else if (worst >= m->coupon_barrier) {
      int64_t a = T * (period + 1) / m->periods, b = T * period / m->periods;
      int64_t ps = a > b ? a - b : 0;
      if (ps < 1) ps = 1;
      accrual += m->coupon_rate / (double)ps;
      o->qualified += 1;
    }
    int all_up = step >= m->call_start;
    for (int f = 0; f < n && all_up; ++f) all_up = spots[f] / m->init[f] >= m->call_barrier;
    if (all_up) {
      ko = 1;
      redemption_time = time;
      o->ko_step = (int)step;
      double due = (period == 0 && m->fixed_first) ? m->coupon_rate : accrual;
      double carry = due > 0.0 ? unpaid : 0.0;
      if (due + carry > 0.0) {
        double df = exp(-m->rate * time);
        coupon_pv += due * df;
        memory_pv += carry * df;
        received = 1;
        o->paid += 1;
      }
      continue;
    }
    int64_t next_period;
    if (step + 1 == T) next_period = m->periods;
    else {
      next_period = ((step + 1) * m->periods) / T;
      if (next_period > m->periods - 1) next_period = m->periods - 1;
    }
    if (step + 1 == T || next_period != period) {
      double due = (period == 0 && m->fixed_first) ? m->coupon_rate : accrual;
      if (due > 0.0) {
        double df = exp(-m->rate * time);
        coupon_pv += due * df;
        memory_pv += unpaid * df;
        received = 1;
        unpaid = 0.0;
        o->paid += 1;
      } else if (m->memory) {
        unpaid += m->coupon_rate;
      }
    }
  }
  /* path close, note.rs:221-258 */
  /* discount factors are libm's in both math modes, as the engine's host tables */
  double funding = exp(-m->rate * redemption_time);
  int hit_ki = final_worst <= m->ki;
  int put_eligible = hit_ki && !ko;
  double put = put_eligible ? fmax(m->strike - final_worst, 0.0) * exp(-m->rate * m->maturity) : 0.0;
  double coupon_nominal = coupon_pv + memory_pv;
  o->worst_final = final_worst;
  o->redemption_time = redemption_time;
  o->put = put;
  o->coupon_pv = coupon_nominal;
  o->memory_pv = memory_pv;
  o->funding = funding;
  o->pv = funding + coupon_nominal - put;
  o->ko = ko;
  o->hit_ki = hit_ki;
  o->put_eligible = put_eligible;
  o->received = received;
}
static void scan_path(const model* m, const double* const* incr, path_out* o) {
  scan_path_cube(m, incr, o, NULL);
}

/* One path of note.rs:81-259. */
static void simulate_path_cube(const model* m, uint64_t path_id, workspace* ws, chacha8* mc, path_out* o,
                               float* cube) {
  path_increments(m, path_id, ws, mc);
  const double* rows[NMAX];
  for (int f = 0; f < m->n; ++f) rows[f] = ws->incr + (size_t)f * (size_t)m->steps;
  scan_path_cube(m, rows, o, cube);
}
static void simulate_path(const model* m, uint64_t path_id, workspace* ws, chacha8* mc, path_out* o) {
  simulate_path_cube(m, path_id, ws, mc, o, NULL);
}

/* ---------------------------------------------------------------- aggregation --------------- */

/* OnlineMoments, note.rs:10-32, plus Chan's pairwise merge for chunked runs. */
typedef struct moments { uint64_t count; double mean, m2; } moments;
static void mom_observe(moments* a, double v) {
  a->count += 1;
  double delta = v - a->mean;
  a->mean += delta / (double)a->count;
  a->m2 += delta * (v - a->mean);
}
static void mom_merge(moments* a, const moments* b) {
  if (b->count == 0) return;
  if (a->count == 0) { *a = *b; return; }
  double n = (double)(a->count + b->count), delta = b->mean - a->mean;
  a->mean += delta * (double)b->count / n;
  a->m2 += b->m2 + delta * delta * (double)a->count * (double)b->count / n;
  a->count += b->count;
}
static double mom_var(const moments* a) { return a->count > 1 ? a->m2 / (double)(a->count - 1) : 0.0; }

typedef struct accum {
  moments pv, ko_funding, ki_put, coupon;
  double put_sum, funding_sum, coupon_sum, coupon_memory_sum;
  uint64_t ko, ki, put_eligible, coupon_paths;
  /* plain FP64 sums in the slot order rg_price_result.path_sums documents (for shard merges) */
  double ps[RG_PATH_SUMS];
  int n_trace;
  rg_trace_event trace[RG_TRACE_EVENT_CAP];
} accum;

static void accum_path(accum* a, const model* m, uint64_t path_id, const path_out* o) {
  if (o->ko) {
    a->ko += 1;
    if (m->trace && a->n_trace < RG_TRACE_EVENT_CAP) {
      a->trace[a->n_trace].path_id = m->first_path + path_id;
      a->trace[a->n_trace].time = o->redemption_time;
      a->n_trace++;
    }
    mom_observe(&a->ko_funding, o->funding);
  }
  if (o->hit_ki) a->ki += 1;
  if (o->put_eligible) a->put_eligible += 1;
  if (o->hit_ki) mom_observe(&a->ki_put, o->put);
  if (o->received) { a->coupon_paths += 1; mom_observe(&a->coupon, o->coupon_pv); }
  double coupon_quote = o->coupon_pv * 10.0, memory_quote = o->memory_pv * 10.0;
  a->funding_sum += o->funding;
  a->put_sum += o->put;
  a->coupon_sum += coupon_quote - memory_quote;
  a->coupon_memory_sum += memory_quote;
  mom_observe(&a->pv, o->pv);
  const double pv1 = o->pv - 1.0;
  a->ps[0] += pv1;
  a->ps[1] += pv1 * pv1;
  if (o->ko) {
    const double f1 = o->funding - 1.0;
    a->ps[2] += f1;
    a->ps[3] += f1 * f1;
    a->ps[12] += 1.0;
  }
  if (o->hit_ki) {
    a->ps[4] += o->put;
    a->ps[5] += o->put * o->put;
    a->ps[13] += 1.0;
  }
  if (o->received) {
    a->ps[6] += o->coupon_pv;
    a->ps[7] += o->coupon_pv * o->coupon_pv;
    a->ps[15] += 1.0;
  }
  a->ps[8] += o->put;
  a->ps[9] += o->funding;
  a->ps[10] += coupon_quote - memory_quote;
  a->ps[11] += memory_quote;
  if (o->put_eligible) a->ps[14] += 1.0;
}

static void accum_merge(accum* a, const accum* b) {
  mom_merge(&a->pv, &b->pv);
  mom_merge(&a->ko_funding, &b->ko_funding);
  mom_merge(&a->ki_put, &b->ki_put);
  mom_merge(&a->coupon, &b->coupon);
  a->put_sum += b->put_sum;
  a->funding_sum += b->funding_sum;
  a->coupon_sum += b->coupon_sum;
  a->coupon_memory_sum += b->coupon_memory_sum;
  a->ko += b->ko;
  a->ki += b->ki;
  a->put_eligible += b->put_eligible;
  a->coupon_paths += b->coupon_paths;
  for (int k = 0; k < RG_PATH_SUMS; ++k) a->ps[k] += b->ps[k];
  for (int i = 0; i < b->n_trace && a->n_trace < RG_TRACE_EVENT_CAP; ++i) a->trace[a->n_trace++] = b->trace[i];
}

/* Aggregates → PriceResult, note.rs:262-372 */
static void finish_result(const accum* a, uint64_t paths, uint64_t seed, rg_price_result* out) {
  memset(out, 0, sizeof *out);
  double P = (double)paths;
  double variance = mom_var(&a->pv);
  double mean_put = a->put_sum / P, mean_funding = a->funding_sum / P;
  double mean_cq = a->coupon_sum / P, mean_mq = a->coupon_memory_sum / P;
  double ko_p = (double)a->ko / P, ki_p = (double)a->ki / P, cp_p = (double)a->coupon_paths / P;
  double total = mean_funding + (mean_cq + mean_mq) / 10.0 - mean_put;
  out->pv = total;
  out->mc_error = sqrt(variance / P);
  out->ki_probability = ki_p;
  out->legs.coupon = mean_cq;
  out->legs.memory_coupon = mean_mq;
  out->legs.down_and_in_put = mean_put;
  out->legs.funding = mean_funding;
  out->legs.total = total;
  rg_transition_stats* s = out->stats;
  s[0].input_count = paths; s[0].output_count = a->ko; s[0].probability = ko_p;
  s[0].mean_payoff = a->ko_funding.mean; s[0].variance_payoff = mom_var(&a->ko_funding);
  s[1].input_count = paths; s[1].output_count = a->ki; s[1].probability = ki_p;
  s[1].mean_payoff = a->ki_put.mean; s[1].variance_payoff = mom_var(&a->ki_put);
  s[2].input_count = paths; s[2].output_count = a->coupon_paths; s[2].probability = cp_p;
  s[2].mean_payoff = a->coupon.mean; s[2].variance_payoff = mom_var(&a->coupon);
  rg_ledger_entry* l = out->ledger;
  l[0].population_before = paths; l[0].population_after = a->ko; l[0].pv_impact = mean_funding * ko_p;
  l[1].population_before = paths - a->ko; l[1].population_after = a->put_eligible; l[1].pv_impact = -mean_put;
  l[2].population_before = paths; l[2].population_after = a->coupon_paths;
  l[2].pv_impact = (mean_cq + mean_mq) / 10.0;
  out->seed = seed;
  out->ko_count = a->ko;
  out->ki_count = a->ki;
  out->put_eligible_count = a->put_eligible;
  out->coupon_path_count = a->coupon_paths;
  out->n_trace_events = a->n_trace;
  memcpy(out->trace_events, a->trace, sizeof(rg_trace_event) * (size_t)a->n_trace);
  memcpy(out->path_sums, a->ps, sizeof a->ps);
}

/* ---------------------------------------------------------------- threading ----------------- */

typedef struct job {
  const model* m;
  uint64_t paths;
  uint64_t n_chunks;
  accum* chunks;
  uint64_t next;
  pthread_mutex_t lock;
} job;

static void* worker(void* arg) {
  job* j = (job*)arg;
  workspace ws;
  ws_alloc(&ws, j->m->n, j->m->steps);
  for (;;) {
    pthread_mutex_lock(&j->lock);
    uint64_t c = j->next++;
    pthread_mutex_unlock(&j->lock);
    if (c >= j->n_chunks) break;
    accum* a = &j->chunks[c];
    memset(a, 0, sizeof *a);
    uint64_t lo = c * CHUNK_PATHS, hi = lo + CHUNK_PATHS < j->paths ? lo + CHUNK_PATHS : j->paths;
    path_out o;
    for (uint64_t p = lo; p < hi; ++p) {
      simulate_path(j->m, p, &ws, NULL, &o);
      accum_path(a, j->m, p, &o);
    }
  }
  ws_free(&ws);
  return NULL;
}

static int32_t price_model(const model* m, uint64_t paths, int threads, accum* total) {
  memset(total, 0, sizeof *total);
  if (threads <= 1 || m->vr == RG_VR_NONE) {
    /* the pseudo-random lane is one sequential stream over all paths */
    workspace ws;
    ws_alloc(&ws, m->n, m->steps);
    chacha8 g;
    pthread_once(&zig_once, zig_init);
    chacha8_seed_u64(&g, m->seed);
    path_out o;
    for (uint64_t p = 0; p < paths; ++p) {
      simulate_path(m, p, &ws, &g, &o);
      accum_path(total, m, p, &o);
    }
    ws_free(&ws);
    return RG_OK;
  }
  job j;
  j.m = m;
  j.paths = paths;
  j.n_chunks = (paths + CHUNK_PATHS - 1) / CHUNK_PATHS;
  j.chunks = (accum*)calloc((size_t)j.n_chunks, sizeof(accum));
  j.next = 0;
  pthread_mutex_init(&j.lock, NULL);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
  for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, worker, &j);
  for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
  for (uint64_t c = 0; c < j.n_chunks; ++c) accum_merge(total, &j.chunks[c]);
  pthread_mutex_destroy(&j.lock);
  free(th);
  free(j.chunks);
  return RG_OK;
}

static int32_t check_lane(const rg_price_request* r) { (void)r; return RG_OK; }

static int32_t price_market(const rg_price_request* r, const rg_market_snapshot* mk,
                            const double* vol_shift, int threads, rg_price_result* out) {
  model m;
  int32_t st = model_init(&m, r, mk, vol_shift);
  if (st) return st;
  accum a;
  st = price_model(&m, r->config.paths, threads, &a);
  if (!st) finish_result(&a, r->config.paths, r->config.seed, out);
  model_free(&m);
  return st;
}

int32_t or_price_put_leg(const rg_price_request* r, int32_t threads, rg_price_result* out) {
  int32_t st = or_validate(r);
  if (st) return st;
  if ((st = check_lane(r))) return st;
  return price_market(r, &r->market, NULL, threads, out);
}

static int32_t run_path_range(const rg_price_request* r, uint64_t first, uint64_t count, rg_path_record* out,
                              float* cube) {
  int32_t st = or_validate(r);
  if (st) return st;
  if ((st = check_lane(r))) return st;
  if (first + count > r->config.paths)
    return fail(RG_ERR_PATH_OUT_OF_RANGE, "path range is outside the configured path count %llu",
                (unsigned long long)r->config.paths);
  model m;
  st = model_init(&m, r, &r->market, NULL);
  if (st) return st;
  workspace ws;
  ws_alloc(&ws, m.n, m.steps);
  path_out o;
  chacha8 g;
  pthread_once(&zig_once, zig_init);
  chacha8_seed_u64(&g, m.seed);
  if (m.vr == RG_VR_NONE) /* advance the sequential stream past the skipped paths */
    for (uint64_t p = 0; p < first; ++p) simulate_path(&m, p, &ws, &g, &o);
  for (uint64_t i = 0; i < count; ++i) {
    uint64_t p = first + i;
    simulate_path_cube(&m, p, &ws, &g, &o, cube ? cube + i * (uint64_t)m.steps * (uint64_t)m.n : NULL);
    if (!out) continue;
    rg_path_record* rec = &out[i];
    memset(rec, 0, sizeof *rec);
    rec->path_id = m.first_path + p;
    rec->rng_seed = r->config.seed;
    rec->sobol_index = m.vr == RG_VR_NONE ? 0 : m.first_path + p + 1;
    rec->worst_final = o.worst_final;
    rec->knocked_out = o.ko;
    rec->ko_step = o.ko_step;
    rec->ko_time = o.ko ? o.redemption_time : NAN;
    rec->ki_hit = o.hit_ki;
    rec->qualified_steps = o.qualified;
    rec->paid_periods = o.paid;
    rec->put_payoff = o.put;
    rec->coupon_pv = o.coupon_pv;
    rec->memory_coupon_pv = o.memory_pv;
    rec->funding = o.funding;
    rec->pv = o.pv;
  }
  ws_free(&ws);
  model_free(&m);
  return RG_OK;
}

int32_t or_run_paths(const rg_price_request* r, uint64_t first, uint64_t count, rg_path_record* out) {
  return run_path_range(r, first, count, out, NULL);
}

/* explain::run_paths with the spot path of every path kept (the replay cube). */
int32_t or_materialize_paths(const rg_price_request* r, uint64_t first, uint64_t count, float* cube,
                             rg_path_record* records) {
  return run_path_range(r, first, count, records, cube);
}

int32_t or_price_scenarios(const rg_price_request* r, const rg_scenario* sc, int32_t n, int32_t threads,
                           rg_price_result* out) {
  int32_t st = or_validate(r);
  if (st) return st;
  if ((st = check_lane(r))) return st;
  for (int32_t i = 0; i < n; ++i) {
    rg_price_request rr = *r;
    rr.market = sc[i].market;
    rr.market.as_of = r->market.as_of;
    if ((st = or_validate(&rr))) return st;
    if ((st = price_market(&rr, &rr.market, sc[i].implied_vol_shift, threads, &out[i]))) return st;
  }
  return RG_OK;
}

/* ============================================================ riga-risk ====================== */

/* validate_configuration, crates/riga-risk/src/lib.rs:338-457 (N-asset: the correlation bump
 * shifts every off-diagonal entry, which is the reference's [0][1]/[1][0] bump at N = 2). */
static int32_t validate_risk(const rg_price_request* r, const rg_central_difference_config* c) {
  if (c->random_number_policy == RG_NO_CRN)
    return fail(RG_ERR_NO_CRN_REJECTED, "central finite differences require CommonRandomNumbers; independent streams are rejected");
  if (!isfinite(c->spot_relative_bump) || c->spot_relative_bump <= 0.0 || c->spot_relative_bump >= 1.0)
    return fail(RG_ERR_INVALID_SPOT_BUMP, "spot_relative_bump must be finite, positive, and less than one");
  if (!isfinite(c->volatility_absolute_bump) || c->volatility_absolute_bump <= 0.0)
    return fail(RG_ERR_INVALID_VOLATILITY_BUMP, "volatility_absolute_bump must be finite and positive");
  if (!isfinite(c->rate_absolute_bump) || c->rate_absolute_bump <= 0.0)
    return fail(RG_ERR_INVALID_RATE_BUMP, "rate_absolute_bump must be finite and positive");
  if (!isfinite(c->correlation_absolute_bump) || c->correlation_absolute_bump <= 0.0)
    return fail(RG_ERR_INVALID_CORRELATION_BUMP, "correlation_absolute_bump must be finite and positive");
  int n = r->market.n_assets;
  if (n < 1 || n > NMAX) return fail(RG_ERR_RISK_INPUT_SHAPE, "spot and volatility arrays must be non-empty and have the same length");
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (i == j) continue;
      double rho = r->market.correlation[i * n + j];
      if (!isfinite(rho) || rho - c->correlation_absolute_bump <= -1.0 || rho + c->correlation_absolute_bump >= 1.0)
        return fail(RG_ERR_INVALID_CORRELATION_BUMP, "correlation up/down scenarios must remain strictly inside (-1, 1)");
    }
  for (int f = 0; f < n; ++f) {
    double s = r->market.spots[f], v = r->market.vols[f];
    if (!isfinite(s) || s <= 0.0) return fail(RG_ERR_INVALID_SPOT_BUMP, "spot[%d] must be finite and positive", f);
    double h = s * c->spot_relative_bump;
    if (!isfinite(h) || h == 0.0 || s - h <= 0.0)
      return fail(RG_ERR_INVALID_SPOT_BUMP, "spot bump for asset %d is not representable and positive", f);
    if (!isfinite(v) || v < c->volatility_absolute_bump)
      return fail(RG_ERR_INVALID_VOLATILITY_BUMP, "volatility[%d] must be finite and at least volatility_absolute_bump", f);
  }
  if (r->config.paths < 2) return fail(RG_ERR_RISK_PATHS_REQUIRED, "at least two paths are required to report Monte Carlo risk uncertainty");
  if (r->n_local_vol) {
    int ok = r->n_local_vol == n;
    for (int f = 0; ok && f < n; ++f) {
      const rg_implied_vol_grid* g = &r->local_vol[f];
      if (g->n_maturities <= 0 || g->n_strikes <= 0) ok = 0;
      for (int i = 0; ok && i < g->n_maturities * g->n_strikes; ++i)
        if (!isfinite(g->vols[i]) || g->vols[i] < c->volatility_absolute_bump) ok = 0;
    }
    if (!ok)
      return fail(RG_ERR_INVALID_VOLATILITY_BUMP, "local-vol surface must align with assets and every implied-vol node must remain non-negative under the down bump");
  }
  return RG_OK;
}

/* Scenario order: base, then per asset {spot+, spot-, vol+, vol-}, rate+, rate-, corr+, corr-
 * (crates/riga-risk/src/lib.rs:117-186, 573-626; scenario_count = 1 + 4n + 4). */
int32_t or_price_risk_batch(const rg_price_request* r, const rg_central_difference_config* c,
                            int32_t threads, rg_batch_risk_report* out) {
  int32_t st = or_validate(r);
  if (st) return st;
  if ((st = validate_risk(r, c))) return st;
  if ((st = check_lane(r))) return st;
  int n = r->market.n_assets;
  int ns = 1 + 4 * n + 4;
  double spots[1 + 4 * NMAX + 4][NMAX], vols[1 + 4 * NMAX + 4][NMAX], shifts[1 + 4 * NMAX + 4][NMAX];
  double corr[1 + 4 * NMAX + 4][NMAX * NMAX];
  rg_scenario sc[1 + 4 * NMAX + 4];
  rg_price_result* res = (rg_price_result*)calloc((size_t)ns, sizeof(rg_price_result));
  for (int s = 0; s < ns; ++s) {
    memcpy(spots[s], r->market.spots, sizeof(double) * (size_t)n);
    memcpy(vols[s], r->market.vols, sizeof(double) * (size_t)n);
    memcpy(corr[s], r->market.correlation, sizeof(double) * (size_t)(n * n));
    memset(shifts[s], 0, sizeof shifts[s]);
    sc[s].market = r->market;
    sc[s].market.spots = spots[s];
    sc[s].market.vols = vols[s];
    sc[s].market.correlation = corr[s];
    sc[s].implied_vol_shift = r->n_local_vol ? shifts[s] : NULL;
  }
  for (int f = 0; f < n; ++f) {
    double h = r->market.spots[f] * c->spot_relative_bump;
    spots[1 + 4 * f][f] += h;
    spots[2 + 4 * f][f] -= h;
    vols[3 + 4 * f][f] += c->volatility_absolute_bump;
    vols[4 + 4 * f][f] += -c->volatility_absolute_bump;
    shifts[3 + 4 * f][f] = c->volatility_absolute_bump;
    shifts[4 + 4 * f][f] = -c->volatility_absolute_bump;
  }
  int ir = 1 + 4 * n;
  sc[ir].market.risk_free_rate += c->rate_absolute_bump;
  sc[ir + 1].market.risk_free_rate += -c->rate_absolute_bump;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (i != j) {
        corr[ir + 2][i * n + j] += c->correlation_absolute_bump;
        corr[ir + 3][i * n + j] += -c->correlation_absolute_bump;
      }
  st = or_price_scenarios(r, sc, ns, threads, res);
  if (st) { free(res); return st; }
  memset(out, 0, sizeof *out);
  out->base = res[0];
  out->scenario_count = (uint64_t)ns;
  out->seed = r->config.seed;
  out->n_assets = n;
  for (int f = 0; f < n; ++f) {
    const rg_price_result *su = &res[1 + 4 * f], *sd = &res[2 + 4 * f], *vu = &res[3 + 4 * f], *vd = &res[4 + 4 * f];
    double h = r->market.spots[f] * c->spot_relative_bump, hv = c->volatility_absolute_bump;
    rg_asset_greeks* g = &out->assets[f];
    g->asset_index = f;
    g->spot_bump = h;
    g->volatility_bump = hv;
    g->delta.value = (su->pv - sd->pv) / (2.0 * h);
    g->delta.mc_error_upper_bound = (su->mc_error + sd->mc_error) / (2.0 * h);
    g->gamma.value = (su->pv - 2.0 * res[0].pv + sd->pv) / (h * h);
    g->gamma.mc_error_upper_bound = (su->mc_error + 2.0 * res[0].mc_error + sd->mc_error) / (h * h);
    g->vega.value = (vu->pv - vd->pv) / (2.0 * hv);
    g->vega.mc_error_upper_bound = (vu->mc_error + vd->mc_error) / (2.0 * hv);
    g->spot_up_pv = su->pv; g->spot_down_pv = sd->pv; g->vol_up_pv = vu->pv; g->vol_down_pv = vd->pv;
    g->spot_up_mc_error = su->mc_error; g->spot_down_mc_error = sd->mc_error;
    g->vol_up_mc_error = vu->mc_error; g->vol_down_mc_error = vd->mc_error;
  }
  /* transition_risk, crates/riga-risk/src/lib.rs:519-554 */
  for (int k = 0; k < RG_N_TRANSITIONS; ++k) {
    double d = 0.0, v = 0.0;
    for (int f = 0; f < n; ++f) {
      double h = out->assets[f].spot_bump, hv = out->assets[f].volatility_bump;
      if (h > 0.0) d += (res[1 + 4 * f].ledger[k].pv_impact - res[2 + 4 * f].ledger[k].pv_impact) / (2.0 * h);
      if (hv > 0.0) v += (res[3 + 4 * f].ledger[k].pv_impact - res[4 + 4 * f].ledger[k].pv_impact) / (2.0 * hv);
    }
    out->transitions[k].pv_impact = res[0].ledger[k].pv_impact;
    out->transitions[k].delta_impact = d;
    out->transitions[k].vega_impact = v;
  }
  out->rate_up_pv = res[ir].pv;
  out->rate_down_pv = res[ir + 1].pv;
  out->correlation_up_pv = res[ir + 2].pv;
  out->correlation_down_pv = res[ir + 3].pv;
  out->rate_bump = c->rate_absolute_bump;
  out->correlation_bump = c->correlation_absolute_bump;
  out->pv_mc_error = res[0].mc_error;
  free(res);
  return RG_OK;
}

/* ============================================================ books ========================== */
/* One universe path set priced for many trades under a common scenario set: the reference's
 * path generation (note.rs:83-106) run once per path for all U universe assets on the universe
 * grid, then, for every (trade, scenario), the reference's step and Phoenix scan
 * (note.rs:129-259) over the first T_j steps of the trade's assets. */

#define BOOK_CHUNK_PATHS 256

typedef struct book_ctx {
  const rg_book_request* r;
  int32_t n_scen; /* S >= 1 */
  const rg_market_snapshot* scen; /* [S] */
  model uni;      /* universe generation model: n = U, steps = universe_steps */
  model* tm;      /* [n_trades * S] scan models */
} book_ctx;

static int32_t book_validate(const rg_book_request* r, const rg_market_snapshot* sc, int32_t n_scen) {
  const rg_market_snapshot* u = &r->universe;
  int U = u->n_assets;
  if (!u->as_of || u->as_of[0] == 0) return fail(RG_ERR_MISSING_AS_OF, "as_of is required");
  if (U < 1 || U > RG_BOOK_MAX_UNIVERSE || !u->spots || !u->vols || !u->dividend_yields || !u->correlation)
    return fail(RG_ERR_INVALID_MARKET_SHAPE, "the universe needs 1..%d assets with aligned arrays", RG_BOOK_MAX_UNIVERSE);
  if (r->config.paths == 0 || r->config.path_block_size == 0)
    return fail(RG_ERR_INVALID_PATHS, "paths and path_block_size must be positive");
  if (r->universe_steps <= 0 || !isfinite(r->universe_maturity_years) || r->universe_maturity_years <= 0.0)
    return fail(RG_ERR_INVALID_SCHEDULE, "universe steps and maturity must be positive and finite");
  if (r->n_trades < 1 || !r->trades) return fail(RG_ERR_INVALID_ARGUMENT, "a book needs at least one trade");
  if (r->config.variance_reduction != RG_VR_SOBOL && r->config.variance_reduction != RG_VR_HALTON)
    return fail(RG_ERR_UNSUPPORTED, "books run the Sobol or Halton lane");
  if (r->config.trace_level != RG_TRACE_OFF)
    return fail(RG_ERR_INVALID_ARGUMENT, "books record no trace events (trace_level must be off)");
  if (n_scen < 0 || (n_scen > 0 && !sc)) return fail(RG_ERR_INVALID_ARGUMENT, "bad scenario list");
  for (int s = 0; s < n_scen; ++s) {
    if (sc[s].n_assets != U || !sc[s].spots || !sc[s].vols || !sc[s].dividend_yields)
      return fail(RG_ERR_INVALID_MARKET_SHAPE, "scenario %d is not a market of the universe", s);
    if (sc[s].correlation && memcmp(sc[s].correlation, u->correlation, sizeof(double) * (size_t)U * (size_t)U) != 0)
      return fail(RG_ERR_INVALID_ARGUMENT, "scenario %d changes the correlation; book scenarios share the base paths", s);
  }
  const double dt = r->universe_maturity_years / (double)r->universe_steps;
  double sub_spots[NMAX], sub_vols[NMAX], sub_q[NMAX], sub_rho[NMAX * NMAX];
  for (int j = 0; j < r->n_trades; ++j) {
    const rg_book_trade* bt = &r->trades[j];
    const rg_phoenix_trade* t = &bt->terms;
    int n = t->n_assets;
    if (n < 1 || n > NMAX || !bt->underlyings)
      return fail(RG_ERR_INVALID_MARKET_SHAPE, "trade %d needs 1..%d underlyings", j, NMAX);
    for (int f = 0; f < n; ++f) {
      int a = bt->underlyings[f];
      if (a < 0 || a >= U) return fail(RG_ERR_INVALID_MARKET_SHAPE, "trade %d underlying %d is outside the universe", j, a);
      for (int g = 0; g < f; ++g)
        if (bt->underlyings[g] == a) return fail(RG_ERR_INVALID_MARKET_SHAPE, "trade %d repeats underlying %d", j, a);
    }
    if (t->steps < 1 || t->steps > r->universe_steps)
      return fail(RG_ERR_INVALID_SCHEDULE, "trade %d steps must be in 1..universe_steps", j);
    if (!(fabs(t->maturity_years - (double)t->steps * dt) <= 1e-12 * t->maturity_years))
      return fail(RG_ERR_INVALID_SCHEDULE, "trade %d maturity must be steps x the universe dt", j);
    /* the reference's own request checks on the trade and its slice of the base market */
    for (int f = 0; f < n; ++f) {
      int a = bt->underlyings[f];
      sub_spots[f] = u->spots[a];
      sub_vols[f] = u->vols[a];
      sub_q[f] = u->dividend_yields[a];
      for (int g = 0; g < n; ++g) sub_rho[f * n + g] = u->correlation[a * U + bt->underlyings[g]];
    }
    rg_price_request q;
    memset(&q, 0, sizeof q);
    q.trade = *t;
    q.market = *u;
    q.market.n_assets = n;
    q.market.spots = sub_spots;
    q.market.vols = sub_vols;
    q.market.dividend_yields = sub_q;
    q.market.correlation = sub_rho;
    q.config = r->config;
    q.as_of = u->as_of;
    int32_t st = or_validate(&q);
    if (st) return st;
  }
  return RG_OK;
}

/* The scan model of trade `t` on underlyings `idx` under universe market `mk`. */
static void book_trade_model(model* m, const rg_phoenix_trade* t, const int32_t* idx,
                             const rg_market_snapshot* mk, double dt) {
  memset(m, 0, sizeof *m);
  m->n = t->n_assets;
  m->steps = t->steps;
  m->periods = t->has_coupon_periods ? t->coupon_periods : 9;
  if (m->periods < 1) m->periods = 1;
  m->call_start = t->has_call_start_step ? t->call_start_step : 0;
  m->dt = dt;
  m->rate = mk->risk_free_rate;
  m->maturity = t->maturity_years;
  for (int f = 0; f < m->n; ++f) {
    m->spots[f] = mk->spots[idx[f]];
    m->init[f] = t->initial_spots[f];
    m->vols[f] = mk->vols[idx[f]];
    m->q[f] = mk->dividend_yields[idx[f]];
  }
  m->call_barrier = t->has_knock_out_barrier ? t->knock_out_barrier : INFINITY;
  m->coupon_barrier = t->has_coupon_barrier ? t->coupon_barrier : INFINITY;
  m->coupon_rate = t->has_coupon_rate ? t->coupon_rate : 0.0;
  m->strike = t->strike;
  m->ki = t->knock_in_barrier;
  m->fixed_first = t->fixed_first_coupon != 0;
  m->memory = t->memory_coupon != 0;
}

static int32_t book_init(book_ctx* b, const rg_book_request* r, const rg_market_snapshot* sc, int32_t n_scen) {
  memset(b, 0, sizeof *b);
  int32_t st = book_validate(r, sc, n_scen);
  if (st) return st;
  b->r = r;
  b->n_scen = n_scen > 0 ? n_scen : 1;
  b->scen = n_scen > 0 ? sc : &r->universe;
  model* u = &b->uni;
  u->n = r->universe.n_assets;
  u->steps = r->universe_steps;
  u->dt = r->universe_maturity_years / (double)r->universe_steps;
  st = or_cholesky(r->universe.correlation, u->n, u->L);
  if (st) return st;
  qmc_init(u, &r->config, (int64_t)u->n * u->steps);
  b->tm = (model*)malloc(sizeof(model) * (size_t)r->n_trades * (size_t)b->n_scen);
  for (int j = 0; j < r->n_trades; ++j)
    for (int s = 0; s < b->n_scen; ++s)
      book_trade_model(&b->tm[(size_t)j * b->n_scen + s], &r->trades[j].terms, r->trades[j].underlyings,
                       &b->scen[s], u->dt);
  return RG_OK;
}

static void book_free(book_ctx* b) {
  model_free(&b->uni);
  free(b->tm);
  b->tm = NULL;
}

/* All (trade, scenario) outcomes of one path: o[j * S + s]. */
static void book_path(const book_ctx* b, uint64_t p, workspace* ws, path_out* o) {
  path_increments(&b->uni, p, ws, NULL);
  const rg_book_request* r = b->r;
  const int64_t TU = b->uni.steps;
  for (int j = 0; j < r->n_trades; ++j) {
    const double* rows[NMAX];
    for (int f = 0; f < r->trades[j].terms.n_assets; ++f)
      rows[f] = ws->incr + (size_t)r->trades[j].underlyings[f] * (size_t)TU;
    for (int s = 0; s < b->n_scen; ++s)
      scan_path(&b->tm[(size_t)j * b->n_scen + s], rows, &o[(size_t)j * b->n_scen + s]);
  }
}

typedef struct book_job {
  const book_ctx* b;
  uint64_t paths, n_chunks, next;
  size_t pairs;
  accum* chunks; /* [n_chunks][pairs] */
  pthread_mutex_t lock;
} book_job;

static void* book_worker(void* arg) {
  book_job* j = (book_job*)arg;
  const book_ctx* b = j->b;
  workspace ws;
  ws_alloc(&ws, b->uni.n, b->uni.steps);
  path_out* o = (path_out*)malloc(sizeof(path_out) * j->pairs);
  for (;;) {
    pthread_mutex_lock(&j->lock);
    uint64_t c = j->next++;
    pthread_mutex_unlock(&j->lock);
    if (c >= j->n_chunks) break;
    accum* a = j->chunks + c * j->pairs;
    memset(a, 0, sizeof(accum) * j->pairs);
    uint64_t lo = c * BOOK_CHUNK_PATHS, hi = lo + BOOK_CHUNK_PATHS < j->paths ? lo + BOOK_CHUNK_PATHS : j->paths;
    for (uint64_t p = lo; p < hi; ++p) {
      book_path(b, p, &ws, o);
      for (size_t k = 0; k < j->pairs; ++k) accum_path(&a[k], &b->tm[k], p, &o[k]);
    }
  }
  free(o);
  ws_free(&ws);
  return NULL;
}

int32_t or_price_book(const rg_book_request* r, const rg_market_snapshot* sc, int32_t n_scen,
                      int32_t threads, rg_price_result* out) {
  book_ctx b;
  int32_t st = book_init(&b, r, sc, n_scen);
  if (st) return st;
  book_job j;
  j.b = &b;
  j.paths = r->config.paths;
  j.pairs = (size_t)r->n_trades * (size_t)b.n_scen;
  j.n_chunks = (j.paths + BOOK_CHUNK_PATHS - 1) / BOOK_CHUNK_PATHS;
  j.chunks = (accum*)calloc((size_t)j.n_chunks * j.pairs, sizeof(accum));
  j.next = 0;
  pthread_mutex_init(&j.lock, NULL);
  int nt = threads > 0 ? threads : 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
  for (int i = 0; i < nt; ++i) pthread_create(&th[i], NULL, book_worker, &j);
  for (int i = 0; i < nt; ++i) pthread_join(th[i], NULL);
  for (size_t k = 0; k < j.pairs; ++k) {
    accum total;
    memset(&total, 0, sizeof total);
    for (uint64_t c = 0; c < j.n_chunks; ++c) accum_merge(&total, &j.chunks[c * j.pairs + k]);
    finish_result(&total, r->config.paths, r->config.seed, &out[k]);
  }
  pthread_mutex_destroy(&j.lock);
  free(th);
  free(j.chunks);
  book_free(&b);
  return RG_OK;
}

int32_t or_book_run_paths(const rg_book_request* r, const rg_market_snapshot* sc, int32_t n_scen,
                          uint64_t first, uint64_t count, rg_path_record* out) {
  book_ctx b;
  int32_t st = book_init(&b, r, sc, n_scen);
  if (st) return st;
  if (first + count > r->config.paths) {
    book_free(&b);
    return fail(RG_ERR_PATH_OUT_OF_RANGE, "path range is outside the configured path count %llu",
                (unsigned long long)r->config.paths);
  }
  size_t pairs = (size_t)r->n_trades * (size_t)b.n_scen;
  workspace ws;
  ws_alloc(&ws, b.uni.n, b.uni.steps);
  path_out* o = (path_out*)malloc(sizeof(path_out) * pairs);
  for (uint64_t i = 0; i < count; ++i) {
    uint64_t p = first + i;
    book_path(&b, p, &ws, o);
    for (size_t k = 0; k < pairs; ++k) {
      rg_path_record* rec = &out[i * pairs + k];
      memset(rec, 0, sizeof *rec);
      rec->path_id = b.uni.first_path + p;
      rec->rng_seed = r->config.seed;
      rec->sobol_index = b.uni.first_path + p + 1;
      rec->worst_final = o[k].worst_final;
      rec->knocked_out = o[k].ko;
      rec->ko_step = o[k].ko_step;
      rec->ko_time = o[k].ko ? o[k].redemption_time : NAN;
      rec->ki_hit = o[k].hit_ki;
      rec->qualified_steps = o[k].qualified;
      rec->paid_periods = o[k].paid;
      rec->put_payoff = o[k].put;
      rec->coupon_pv = o[k].coupon_pv;
      rec->memory_coupon_pv = o[k].memory_pv;
      rec->funding = o[k].funding;
      rec->pv = o[k].pv;
    }
  }
  free(o);
  ws_free(&ws);
  book_free(&b);
  return RG_OK;
}

/* ============================================================ PathCube ======================= */
/* generate_correlated_block, crates/riga-engine/src/pathcube.rs:37-66: per (path, time) draw
 * `factors` normals of the one ChaCha8 stream, y = L·z, store (f32)y. */
void or_generate_correlated_block(uint64_t seed, int64_t paths, int64_t times, int32_t factors,
                                  const double* chol, float* out) {
  pthread_once(&zig_once, zig_init);
  chacha8 g;
  chacha8_seed_u64(&g, seed);
  double z[RG_BOOK_MAX_UNIVERSE], y[RG_BOOK_MAX_UNIVERSE];
  for (int64_t p = 0; p < paths; ++p)
    for (int64_t t = 0; t < times; ++t) {
      for (int f = 0; f < factors; ++f) z[f] = zig_normal(&g);
      chol_apply(chol, factors, z, y);
      for (int f = 0; f < factors; ++f) out[(p * times + t) * factors + f] = (float)y[f];
    }
}

/* gbm_evolve, crates/riga-engine/src/pathcube.rs:146-187 (FP64 log-space, f32 output). */
int32_t or_gbm_evolve(const double* s0, const double* vols, double rate, const double* q, int32_t factors,
                      double dt, const float* block, int64_t paths, int64_t times, float* out) {
  if (factors < 1) return fail(RG_ERR_SHAPE_MISMATCH, "s0, vols and dividend_yields must have equal length");
  double sqrt_dt = sqrt(dt);
  for (int64_t p = 0; p < paths; ++p)
    for (int f = 0; f < factors; ++f) {
      double log_s = log(s0[f]);
      double drift = (rate - q[f] - 0.5 * vols[f] * vols[f]) * dt;
      double diffusion = vols[f] * sqrt_dt;
      for (int64_t i = 0; i < times; ++i) {
        int64_t at = (p * times + i) * factors + f;
        log_s += drift + diffusion * (double)block[at];
        out[at] = (float)exp(log_s);
      }
    }
  return RG_OK;
}
