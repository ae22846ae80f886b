// potentials.cuh -- pair and EAM functionals on the device, in FP64 (reference formulas)
// and FP32 (mixed path).
//
//   LennardJones   plugins/lennardjones.cc:53-67     p = {sigma, epsilon, cutoff}
//   SuttonChen     plugins/suttonchen.cc:73-95       p = {e, a, n, m, c, cutoff}
//   FinnisSinclair plugins/finnissinclair.cc:75-113  p = {c0, c1, c2, A, B, c, d}
//   FS-ext         plugins/finnissinclair-ext.cc:85-128 p = {c0, c1, c2, c3, c4, A, B, c, d}
//
// The force of a pair is returned as a scalar g with F_i = g * r_ij (r_ij = x_j - x_i), so
// the virial term -r_ij.F_i is -g*r^2 and the stress term -r_ij[a] F_i[b] is -g r_a r_b.
#pragma once

#include "device.cuh"

namespace gbmd {

__device__ __forceinline__ bool applies_to(int spc_sum, int s1, int s2) {
  return (spc_sum < 0) || ((s1 + s2) == spc_sum);  // liblpmd/simulation/potential.cc:25-27
}

__device__ __forceinline__ double ipow_d(double x, int n) {
  double r = 1.0, b = x;
  while (n > 0) {
    if (n & 1) r = dmul(r, b);
    b = dmul(b, b);
    n >>= 1;
  }
  return r;
}

__device__ __forceinline__ float ipow_f(float x, int n) {
  float r = 1.0f, b = x;
  while (n > 0) {
    if (n & 1) r *= b;
    b *= b;
    n >>= 1;
  }
  return r;
}

// ------------------------------------------------------------------------------------------
// FP64
// ------------------------------------------------------------------------------------------

// LennardJones pairForce/pairEnergy: ff = -48 (eps/r^2) (s^12 - 0.5 s^6), E = 4 eps (s^12 - s^6)
// with s^6 = (sigma^2/r^2)^3.
__device__ __forceinline__ void lj_pair64(const PotParams& P, double r2, double& g, double& e) {
  const double sigma = P.p[0], eps = P.p[1];
  double x = ddiv(dmul(sigma, sigma), r2);
  double r6 = dmul(dmul(x, x), x);
  double r12 = dmul(r6, r6);
  g = dmul(dmul(-48.0, ddiv(eps, r2)), dsub(r12, dmul(0.5, r6)));
  e = dmul(dmul(4.0, eps), dsub(r12, r6));
}

// FastLJ pairEnergy / pairForce (plugins/fastlj.cc:56-73): the tabulated LJ values of bin
// k = floor(bins r / cutoff) (no interpolation).  k is clamped to the last bin, which a distance
// that rounds to the cutoff would otherwise pass (the reference reads past its table there).
__device__ __forceinline__ void fastlj_pair64(const PotParams& P, double r2, double& g, double& e) {
  const long bins = (long)P.p[3];
  long k = (long)floor(ddiv(dmul((double)bins, sqrt(r2)), P.cutoff));
  if (k > bins - 1) k = bins - 1;
  e = P.tab[k];
  g = P.tab[bins + k];
}

// rhoij(r) for the EAM density pass.
__device__ __forceinline__ double eam_rho64(const PotParams& P, double r) {
  if (P.kind == POT_GUPTA) {  // plugins/gupta.cc:56: exp(-2 q (r - r0) / r0)
    const double r0 = P.p[1], q = P.p[4];
    return exp(ddiv(dmul(dmul(-2.0, q), dsub(r, r0)), r0));
  }
  if (P.kind == POT_SC) {
    double ir = ddiv(1.0, r);
    double pw = (P.int_m >= 0) ? ipow_d(ir, P.int_m) : pow(ir, P.p[3]);
    return dmul(P.am, pw);
  } else if (P.kind == POT_FS) {
    const double B = P.p[4], d = P.p[6];
    if (r <= d) {
      double rd = dsub(r, d);
      return dmul(dmul(rd, rd), dadd(1.0, ddiv(dmul(B, rd), d)));
    }
    return 0.0;
  } else {
    const double B = P.p[6], d = P.p[8];
    if (r <= d) {
      double rd = dsub(r, d);
      return dmul(dmul(rd, rd), dadd(1.0, dmul(dmul(dmul(B, B), rd), rd)));
    }
    return 0.0;
  }
}

// Embedding F(rho) and 1/sqrt(rho) (the per-atom factor of ManyBodies).
__device__ __forceinline__ void eam_embed64(const PotParams& P, double rho, double& F, double& phi) {
  double sq = sqrt(rho);
  if (P.kind == POT_SC)
    F = dmul(dmul(-P.p[4], P.p[0]), sq);
  else if (P.kind == POT_FS || P.kind == POT_GUPTA)  // FS: -A sqrt(rho); Gupta: -B sqrt(rho)
    F = dmul(-P.p[3], sq);
  else
    F = dmul(-P.p[5], sq);
  phi = ddiv(1.0, sq);
}

// Pair energy V(r) and the scalar s with PairForce + ManyBodies = s * r^ (r^ = r_ij / r).
__device__ __forceinline__ void eam_pair64(const PotParams& P, double r, double phi_i, double phi_j,
                                           double& s, double& e) {
  if (P.kind == POT_GUPTA) {
    // plugins/gupta.cc:54,60-70: V = A exp(-p (r - r0) / r0), PairForce = -(A p / r0) exp(..),
    // ManyBodies = (B q / r0) (1/sqrt(rho_i) + 1/sqrt(rho_j)) exp(-2 q (r - r0) / r0)
    const double A = P.p[0], r0 = P.p[1], pp = P.p[2], B = P.p[3], q = P.p[4];
    const double dr = dsub(r, r0);
    const double ex = exp(ddiv(dmul(-pp, dr), r0));
    e = dmul(A, ex);
    const double pf = dmul(-ddiv(dmul(A, pp), r0), ex);
    const double mb = dmul(dmul(ddiv(dmul(B, q), r0), dadd(phi_i, phi_j)), exp(ddiv(dmul(dmul(-2.0, q), dr), r0)));
    s = dadd(pf, mb);
  } else if (P.kind == POT_SC) {
    const double eps = P.p[0], n = P.p[2], m = P.p[3], c = P.p[4];
    double ir = ddiv(1.0, r);
    double irn = (P.int_n >= 0) ? ipow_d(ir, P.int_n) : pow(ir, n);
    double irm1 = (P.int_m >= 0) ? ipow_d(ir, P.int_m + 1) : pow(ir, m + 1);
    e = dmul(dmul(eps, P.an), irn);
    double pf = dmul(dmul(dmul(-n, eps), P.an), dmul(irn, ir));
    double mb = dmul(dmul(dmul(dmul(dmul(dmul(0.5, m), c), eps), dadd(phi_i, phi_j)), P.am), irm1);
    s = dadd(pf, mb);
  } else if (P.kind == POT_FS) {
    const double c0 = P.p[0], c1 = P.p[1], c2 = P.p[2], A = P.p[3], B = P.p[4], c = P.p[5], d = P.p[6];
    double pf = 0.0, mb = 0.0;
    e = 0.0;
    if (r <= c) {
      double rc = dsub(r, c);
      double poly = dadd(dadd(c0, dmul(c1, r)), dmul(dmul(c2, r), r));
      e = dmul(dmul(rc, rc), poly);
      double t1 = dmul(dmul(2.0, rc), poly);
      double t2 = dmul(dmul(rc, rc), dadd(c1, dmul(dmul(2.0, c2), r)));
      pf = dadd(t1, t2);
    }
    if (r <= d) {
      double rd = dsub(r, d);
      double t1 = ddiv(dmul(dadd(phi_i, phi_j), A), 2.0);
      double t2 = dadd(dmul(2.0, rd), ddiv(dmul(dmul(dmul(3.0, B), rd), rd), d));
      mb = dmul(-t1, t2);
    }
    s = dadd(pf, mb);
  } else {
    const double c0 = P.p[0], c1 = P.p[1], c2 = P.p[2], c3 = P.p[3], c4 = P.p[4];
    const double A = P.p[5], B = P.p[6], c = P.p[7], d = P.p[8];
    double pf = 0.0, mb = 0.0;
    e = 0.0;
    if (r <= c) {
      double r2 = dmul(r, r);
      double rc = dsub(r, c);
      double poly = dadd(dadd(dadd(dadd(c0, dmul(c1, r)), dmul(c2, r2)), dmul(dmul(c3, r2), r)),
                         dmul(dmul(c4, r2), r2));
      e = dmul(dmul(rc, rc), poly);
      double t1 = dmul(dmul(2.0, rc), poly);
      double dp = dadd(dadd(dadd(c1, dmul(dmul(2.0, c2), r)), dmul(dmul(3.0, c3), r2)),
                       dmul(dmul(dmul(4.0, c4), r2), r));
      double t2 = dmul(dmul(dp, rc), rc);
      pf = dadd(t1, t2);
    }
    if (r <= d) {
      double rd = dsub(r, d);
      double t1 = dmul(dmul(A, 0.5), dadd(phi_i, phi_j));
      double t2 = dadd(dmul(2.0, rd), dmul(dmul(dmul(dmul(dmul(4.0, B), B), rd), rd), rd));
      mb = dmul(-t1, t2);
    }
    s = dadd(pf, mb);
  }
}

// ------------------------------------------------------------------------------------------
// FP32 (mixed path).  Constants in P.f:
//   LJ: f[0]=sigma^2, f[1]=48 eps, f[2]=24 eps, f[3]=4 eps, f[4]=sigma^2 - f[0]
//   SC: f[0]=e*an, f[1]=-n*e*an, f[2]=0.5*m*c*e*am, f[3]=am
//   FS/FSX: f[0..4]=c0..c4, f[5]=A, f[6]=B, f[7]=c, f[8]=d
//   Gupta: f[0]=A, f[1]=-p/r0, f[2]=-A p/r0, f[3]=B q/r0, f[4]=-2q/r0, f[5]=r0
//   all EAM, set per launch: f[14] = the factor the density pass applies to the embedding factor
//   it stores beside the position (f[2] for the folded Sutton-Chen form, else 1)
// ------------------------------------------------------------------------------------------

// g with F_i = g * r_ij, and the pair energy e; inv = 1/r^2.  sigma^2 enters as the double-float
// f[0] + f[4]: its FP32 rounding would scale (sigma/r)^12 and (sigma/r)^6 differently for every
// pair alike, a bias the virial (where the two terms cancel) amplifies.  (The hardware reciprocal
// showed no such bias: refining it by a Newton step changed no error measurably.)
__device__ __forceinline__ void lj_pair32(const PotParams& P, float inv, float& g, float& e) {
  float x = fmaf(P.f[0], inv, P.f[4] * inv);  // one rounding of (f[0] + f[4]) * inv
  float r6 = x * x * x;
  g = -inv * r6 * fmaf(P.f[1], r6, -P.f[2]);
  e = r6 * fmaf(P.f[3], r6, -P.f[3]);
}

// lj_pair32 for two list entries, the products of variables as packed FP32 pairs and the
// products with the parameters as scalars (their operands stay in the constant bank); every
// value is bitwise the scalar form's.  The sign of g is carried by the bracket: (inv r6)
// (f2 - f1 r6) = (-inv r6)(f1 r6 - f2) exactly, rounding being symmetric.
__device__ __forceinline__ void lj_pair32_x2(const PotParams& P, float inva, float invb, float& ga, float& gb,
                                             float& ea, float& eb) {
  const float xa = fmaf(P.f[0], inva, P.f[4] * inva), xb = fmaf(P.f[0], invb, P.f[4] * invb);
  const f32x2 x = f2_pack(xa, xb);
  const f32x2 r6 = f2_mul(f2_mul(x, x), x);
  float r6a, r6b;
  f2_unpack(r6, r6a, r6b);
  const f32x2 nt = f2_pack(fmaf(-P.f[1], r6a, P.f[2]), fmaf(-P.f[1], r6b, P.f[2]));
  f2_unpack(f2_mul(f2_mul(f2_pack(inva, invb), r6), nt), ga, gb);
  const f32x2 u = f2_pack(fmaf(P.f[3], r6a, -P.f[3]), fmaf(P.f[3], r6b, -P.f[3]));
  f2_unpack(f2_mul(r6, u), ea, eb);
}

__device__ __forceinline__ float eam_rho32(const PotParams& P, float r2) {
  if (P.kind == POT_GUPTA) return expf(P.f[4] * (r2 * rsqrt_nr(r2) - P.f[5]));
  if (P.kind == POT_SC) {
    if (P.int_m >= 0 && (P.int_m & 1) == 0) return P.f[3] * ipow_f(__frcp_rn(r2), P.int_m >> 1);
    float ir = rsqrt_nr(r2);
    return P.f[3] * ((P.int_m >= 0) ? ipow_f(ir, P.int_m) : __powf(ir, (float)P.p[3]));
  } else {
    float r = sqrtf(r2);
    const float B = P.f[6], d = P.f[8];
    if (r <= d) {
      float rd = r - d;
      if (P.kind == POT_FS) return rd * rd * (1.0f + B * rd / d);
      return rd * rd * (1.0f + B * B * rd * rd);
    }
    return 0.0f;
  }
}

// x^N for a compile-time N by repeated squaring (straight-line code).
template <int N>
__device__ __forceinline__ float ipow_c(float x) {
  if constexpr (N == 0) {
    return 1.0f;
  } else if constexpr (N == 1) {
    return x;
  } else if constexpr (N % 2 == 0) {
    const float h = ipow_c<N / 2>(x);
    return h * h;
  } else {
    return x * ipow_c<N - 1>(x);
  }
}
// s with F_i = s * r_ij (note: r_ij, not r^) and pair energy e.
__device__ __forceinline__ void eam_pair32(const PotParams& P, float r2, float phi_i, float phi_j, float& s,
                                           float& e) {
  if (P.kind == POT_GUPTA) {
    const float ir = rsqrt_nr(r2), dr = r2 * ir - P.f[5];
    const float ex = expf(P.f[1] * dr);
    e = P.f[0] * ex;
    s = (P.f[2] * ex + P.f[3] * (phi_i + phi_j) * expf(P.f[4] * dr)) * ir;
  } else if (P.kind == POT_SC) {
    float ir = rsqrt_nr(r2);
    float irn = (P.int_n >= 0) ? ipow_f(ir, P.int_n) : __powf(ir, (float)P.p[2]);
    float irm1 = (P.int_m >= 0) ? ipow_f(ir, P.int_m + 1) : __powf(ir, (float)P.p[3] + 1.0f);
    e = P.f[0] * irn;
    s = (P.f[1] * irn * ir + P.f[2] * (phi_i + phi_j) * irm1) * ir;
  } else {
    float r = r2 * rsqrt_nr(r2);
    float ir = 1.0f / r;
    const float c0 = P.f[0], c1 = P.f[1], c2 = P.f[2], c3 = P.f[3], c4 = P.f[4];
    const float A = P.f[5], B = P.f[6], c = P.f[7], d = P.f[8];
    float pf = 0.0f, mb = 0.0f;
    e = 0.0f;
    if (r <= c) {
      float rc = r - c;
      float poly, dp;
      if (P.kind == POT_FS) {
        poly = c0 + c1 * r + c2 * r * r;
        dp = c1 + 2.0f * c2 * r;
      } else {
        float rr = r * r;
        poly = c0 + c1 * r + c2 * rr + c3 * rr * r + c4 * rr * rr;
        dp = c1 + 2.0f * c2 * r + 3.0f * c3 * rr + 4.0f * c4 * rr * r;
      }
      e = rc * rc * poly;
      pf = 2.0f * rc * poly + rc * rc * dp;
    }
    if (r <= d) {
      float rd = r - d;
      float t1 = 0.5f * A * (phi_i + phi_j);
      float t2 = (P.kind == POT_FS) ? (2.0f * rd + 3.0f * B * rd * rd / d) : (2.0f * rd + 4.0f * B * B * rd * rd * rd);
      mb = -t1 * t2;
    }
    s = (pf + mb) * ir;
  }
}

// Sutton-Chen with the exponents n = N, m = M known at compile time (the kernels are
// instantiated for the common pairs); N = M = 0 selects the run-time forms above.
template <int M>
__device__ __forceinline__ float eam_rho32_t(const PotParams& P, float r2) {
  if constexpr (M > 0) {
    if constexpr (M % 2 == 0)
      return P.f[3] * ipow_c<M / 2>(rcp_nr(r2));
    else
      return P.f[3] * ipow_c<M>(rsqrt_nr(r2));
  } else {
    return eam_rho32(P, r2);
  }
}

// Sutton-Chen with compile-time n = N, m = M and the many-body prefactor folded into the
// embedding factors: qi = f[2] / sqrt(rho_i) (and qj), so s = f[1] r^-(N+2) + (qi + qj) r^-(M+2)
// and e = f[0] r^-N, every power built from 1/r^2 and one refined 1/r.
template <int N, int M>
__device__ __forceinline__ void eam_sc_pair32_q(const PotParams& P, float r2, float qi, float qj, float& s,
                                                float& e) {
  static_assert(M % 2 == 0, "the folded form takes even m");
  const float ir = rsqrt_nr(r2);
  const float inv = ir * ir;
  const float pm = ipow_c<(M + 2) / 2>(inv);                                  // r^-(M+2)
  const float pn = (N % 2 == 0) ? ipow_c<N / 2>(inv) : ipow_c<N / 2>(inv) * ir;  // r^-N
  e = P.f[0] * pn;
  s = fmaf(P.f[1], pn * inv, (qi + qj) * pm);
}

// x^N of a packed pair by the same repeated squaring as ipow_c.
template <int N>
__device__ __forceinline__ f32x2 ipow_c_x2(f32x2 x) {
  if constexpr (N == 1) {
    return x;
  } else if constexpr (N % 2 == 0) {
    const f32x2 h = ipow_c_x2<N / 2>(x);
    return f2_mul(h, h);
  } else {
    return f2_mul(x, ipow_c_x2<N - 1>(x));
  }
}

// eam_sc_pair32_q for two list entries (qja, qjb: the neighbours' factors), bitwise the same
// values: the products of variables packed, the products with constants scalar.
template <int N, int M>
__device__ __forceinline__ void eam_sc_pair32_q_x2(const PotParams& P, float r2a, float r2b, float qi, float qja,
                                                   float qjb, float& sa, float& sb, float& ea, float& eb) {
  static_assert(M % 2 == 0 && M >= 2 && N >= 2, "the folded form takes even m");
  // rsqrt_nr per lane: y = rsqrt(x); e = 1 - (x y) y; y + (y/2) e
  const float ya = rsqrtf(r2a), yb = rsqrtf(r2b);
  const f32x2 y = f2_pack(ya, yb);
  float pa, pb;
  f2_unpack(f2_mul(f2_pack(r2a, r2b), y), pa, pb);
  const f32x2 e = f2_pack(fmaf(-pa, ya, 1.0f), fmaf(-pb, yb, 1.0f));
  const f32x2 ir = f2_fma(f2_pack(0.5f * ya, 0.5f * yb), e, y);
  const f32x2 inv = f2_mul(ir, ir);
  const f32x2 pm = ipow_c_x2<(M + 2) / 2>(inv);                                            // r^-(M+2)
  const f32x2 pn = (N % 2 == 0) ? ipow_c_x2<N / 2>(inv) : f2_mul(ipow_c_x2<N / 2>(inv), ir);  // r^-N
  float pna, pnb;
  f2_unpack(pn, pna, pnb);
  ea = P.f[0] * pna;
  eb = P.f[0] * pnb;
  float pia, pib, qa, qb;
  f2_unpack(f2_mul(pn, inv), pia, pib);
  f2_unpack(f2_mul(f2_add(f2_pack(qi, qi), f2_pack(qja, qjb)), pm), qa, qb);
  sa = fmaf(P.f[1], pia, qa);
  sb = fmaf(P.f[1], pib, qb);
}

template <int N, int M>
__device__ __forceinline__ void eam_pair32_t(const PotParams& P, float r2, float phi_i, float phi_j, float& s,
                                             float& e) {
  if constexpr (N > 0) {
    const float ir = rsqrt_nr(r2);
    const float irm1 = ipow_c<M + 1>(ir);
    const float irn = ipow_c<N>(ir);
    e = P.f[0] * irn;
    s = (P.f[1] * irn * ir + P.f[2] * (phi_i + phi_j) * irm1) * ir;
  } else {
    eam_pair32(P, r2, phi_i, phi_j, s, e);
  }
}

}  // namespace gbmd
