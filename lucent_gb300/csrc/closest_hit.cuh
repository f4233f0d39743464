// Closest-hit decisions of the reference's CPU intersector, reproduced on the
// GPU: f32 tests with proven error bounds decide every case they can, and the
// rest are recomputed in binary64 with the reference's exact operation order.
#pragma once
#include "common.cuh"

namespace lucent {

// Inputs whose f32 images stay far from overflow and underflow, so the error
// bounds below hold: |coordinate| <= 2^30 and 2^-30 <= |dir component| <= 2^30.
constexpr float kSafeCoord = 1073741824.0f;  // 2^30
constexpr float kSafeDirLo = 9.3132257e-10f; // 2^-30

LUCENT_DEV bool safe_ray(float3 o, float3 d) {
  const bool fo = fabsf(o.x) <= kSafeCoord && fabsf(o.y) <= kSafeCoord && fabsf(o.z) <= kSafeCoord;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  const bool fd = ax >= kSafeDirLo && ay >= kSafeDirLo && az >= kSafeDirLo && ax <= kSafeCoord &&
                  ay <= kSafeCoord && az <= kSafeCoord;
  return fo && fd;
}

// Per-ray f32 state. `inv` is the correctly rounded f32 reciprocal.
struct Ray32 {
  float3 o, d, inv;
  int negx, negy, negz;  // sign of inv: which slab bound is the entry
};

LUCENT_DEV Ray32 make_ray32(float3 o, float3 d) {
  Ray32 r;
  r.o = o;
  r.d = d;
  r.inv = make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
  r.negx = r.inv.x < 0.f;
  r.negy = r.inv.y < 0.f;
  r.negz = r.inv.z < 0.f;
  return r;
}

// Slab-test classification against the reference's binary64 slab test
// (src/math/aabb.ts:84-98) with running closest `c` given as f32 bounds.
enum SlabClass { kCulled = 0, kPass = 1, kAmbiguous = 2 };

// t = (b - o) * inv computed with 3 roundings in f32 and ~3 in f64; the two
// differ by at most 4 ulp(f32) relative plus an absolute floor for results
// that fall into the f32 subnormal range.
constexpr float kSlabRel = 2.384185791e-07f;  // 2^-22
constexpr float kAbsFloor = 7.8886091e-31f;   // 2^-100

LUCENT_DEV float slab_t(float b, float o, float inv) { return __fmul_rn(__fsub_rn(b, o), inv); }
LUCENT_DEV float widen(float t) { return __fmaf_ru(fabsf(t), kSlabRel, kAbsFloor); }

// Same classification; also returns an upper bound on the reference's entry
// distance max(0, entries), which decides later re-tests after `c` shrinks.
LUCENT_DEV SlabClass classify_slab_e(const Ray32& r, float4 mn, float4 mx, float c_lo, float c_hi, float& ehi) {
  const float ax0 = slab_t(mn.x, r.o.x, r.inv.x), ax1 = slab_t(mx.x, r.o.x, r.inv.x);
  const float ay0 = slab_t(mn.y, r.o.y, r.inv.y), ay1 = slab_t(mx.y, r.o.y, r.inv.y);
  const float az0 = slab_t(mn.z, r.o.z, r.inv.z), az1 = slab_t(mx.z, r.o.z, r.inv.z);
  const float ex = r.negx ? ax1 : ax0, xx = r.negx ? ax0 : ax1;
  const float ey = r.negy ? ay1 : ay0, xy = r.negy ? ay0 : ay1;
  const float ez = r.negz ? az1 : az0, xz = r.negz ? az0 : az1;
  const float wex = widen(ex), wey = widen(ey), wez = widen(ez);
  const float wxx = widen(xx), wxy = widen(xy), wxz = widen(xz);
  const float ex_hi = ex + wex, ey_hi = ey + wey, ez_hi = ez + wez;
  const float xx_lo = xx - wxx, xy_lo = xy - wxy, xz_lo = xz - wxz;
  const float emax_lo = fmaxf(fmaxf(ex - wex, ey - wey), fmaxf(ez - wez, 0.f));
  const float xmin_hi = fminf(fminf(xx + wxx, xy + wxy), fminf(xz + wxz, c_hi));
  ehi = fmaxf(fmaxf(ex_hi, ey_hi), fmaxf(ez_hi, 0.f));
  if (xmin_hi < emax_lo) return kCulled;
  const bool okx = xx_lo >= fmaxf(fmaxf(ey_hi, ez_hi), 0.f);
  const bool oky = xy_lo >= fmaxf(fmaxf(ex_hi, ez_hi), 0.f);
  const bool okz = xz_lo >= fmaxf(fmaxf(ex_hi, ey_hi), 0.f);
  return (okx && oky && okz && c_lo >= ehi) ? kPass : kAmbiguous;
}

LUCENT_DEV SlabClass classify_slab(const Ray32& r, float4 mn, float4 mx, float c_lo, float c_hi) {
  // Entry/exit per axis: after the reference's swap the entry is the bound the
  // ray meets first, fixed by the sign of the direction.
  const float ax0 = slab_t(mn.x, r.o.x, r.inv.x), ax1 = slab_t(mx.x, r.o.x, r.inv.x);
  const float ay0 = slab_t(mn.y, r.o.y, r.inv.y), ay1 = slab_t(mx.y, r.o.y, r.inv.y);
  const float az0 = slab_t(mn.z, r.o.z, r.inv.z), az1 = slab_t(mx.z, r.o.z, r.inv.z);
  const float ex = r.negx ? ax1 : ax0, xx = r.negx ? ax0 : ax1;
  const float ey = r.negy ? ay1 : ay0, xy = r.negy ? ay0 : ay1;
  const float ez = r.negz ? az1 : az0, xz = r.negz ? az0 : az1;
  const float wex = widen(ex), wey = widen(ey), wez = widen(ez);
  const float wxx = widen(xx), wxy = widen(xy), wxz = widen(xz);
  const float ex_lo = ex - wex, ey_lo = ey - wey, ez_lo = ez - wez;
  const float ex_hi = ex + wex, ey_hi = ey + wey, ez_hi = ez + wez;
  const float xx_lo = xx - wxx, xy_lo = xy - wxy, xz_lo = xz - wxz;
  const float xx_hi = xx + wxx, xy_hi = xy + wxy, xz_hi = xz + wxz;
  // Culled for sure: some exit (or c) lies below some entry (or 0). A same-axis
  // pair can never qualify, since exit >= entry on one axis in both precisions.
  const float emax_lo = fmaxf(fmaxf(ex_lo, ey_lo), fmaxf(ez_lo, 0.f));
  const float xmin_hi = fminf(fminf(xx_hi, xy_hi), fminf(xz_hi, c_hi));
  if (xmin_hi < emax_lo) return kCulled;
  // Passes for sure: every cross-axis pair, every exit vs 0 and c vs every
  // entry is ordered with margin. Same-axis pairs are exact (flat boxes).
  const bool okx = xx_lo >= fmaxf(fmaxf(ey_hi, ez_hi), 0.f);
  const bool oky = xy_lo >= fmaxf(fmaxf(ex_hi, ez_hi), 0.f);
  const bool okz = xz_lo >= fmaxf(fmaxf(ex_hi, ey_hi), 0.f);
  const bool okc = c_lo >= fmaxf(fmaxf(ex_hi, ey_hi), ez_hi);
  return (okx && oky && okz && okc) ? kPass : kAmbiguous;
}

// Moller-Trumbore f32 prefilter. Returns false only when the reference's
// binary64 intersectTriangle (src/math/ray.ts:22-45) with (tMin, c) certainly
// rejects. Every numerator is bounded by 2^-19 x its absolute-value
// evaluation (>= 4x the worst-case rounding of either precision: at most 8
// roundings deep) plus an absolute floor.
constexpr float kMtRel = 1.9073486e-06f;  // 2^-19

LUCENT_DEV bool mt_candidate(const Ray32& r, float4 a, float4 b, float4 c3, float tmin_lo, float c_hi) {
  const float3 e1 = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
  const float3 e2 = make_float3(c3.x - a.x, c3.y - a.y, c3.z - a.z);
  const float3 d = r.d;
  const float3 p = make_float3(d.y * e2.z - d.z * e2.y, d.z * e2.x - d.x * e2.z, d.x * e2.y - d.y * e2.x);
  const float det = e1.x * p.x + e1.y * p.y + e1.z * p.z;
  const float3 s = make_float3(r.o.x - a.x, r.o.y - a.y, r.o.z - a.z);
  const float U = s.x * p.x + s.y * p.y + s.z * p.z;
  const float3 q = make_float3(s.y * e1.z - s.z * e1.y, s.z * e1.x - s.x * e1.z, s.x * e1.y - s.y * e1.x);
  const float V = d.x * q.x + d.y * q.y + d.z * q.z;
  const float T = e2.x * q.x + e2.y * q.y + e2.z * q.z;
  // Absolute-value evaluations.
  const float3 ad = make_float3(fabsf(d.x), fabsf(d.y), fabsf(d.z));
  const float3 ae1 = make_float3(fabsf(e1.x), fabsf(e1.y), fabsf(e1.z));
  const float3 ae2 = make_float3(fabsf(e2.x), fabsf(e2.y), fabsf(e2.z));
  const float3 as = make_float3(fabsf(s.x), fabsf(s.y), fabsf(s.z));
  const float3 ap = make_float3(ad.y * ae2.z + ad.z * ae2.y, ad.z * ae2.x + ad.x * ae2.z, ad.x * ae2.y + ad.y * ae2.x);
  const float3 aq = make_float3(as.y * ae1.z + as.z * ae1.y, as.z * ae1.x + as.x * ae1.z, as.x * ae1.y + as.y * ae1.x);
  const float eD = fmaf(ae1.x * ap.x + ae1.y * ap.y + ae1.z * ap.z, kMtRel, kAbsFloor);
  const float eU = fmaf(as.x * ap.x + as.y * ap.y + as.z * ap.z, kMtRel, kAbsFloor);
  const float eV = fmaf(ad.x * aq.x + ad.y * aq.y + ad.z * aq.z, kMtRel, kAbsFloor);
  const float eT = fmaf(ae2.x * aq.x + ae2.y * aq.y + ae2.z * aq.z, kMtRel, kAbsFloor);

  const float A = fabsf(det);
  if (A + eD < 9.9e-13f) return false;  // |det| < 1e-12 for sure
  if (A <= eD) return true;             // sign of det unknown: decide in f64
  const float sg = det < 0.f ? -1.f : 1.f;
  const float Ua = U * sg, Va = V * sg, Ta = T * sg;
  const float Ahi = A + eD, Alo = A - eD;
  if (Ua + eU < 0.f) return false;              // u < 0
  if (Ua - eU > Ahi) return false;              // u > 1
  if (Va + eV < 0.f) return false;              // v < 0
  if (Ua + Va - (eU + eV) > Ahi) return false;  // u + v > 1
  if (Ta + eT < 0.f) return false;              // t < 0 <= tMin
  if (Ta + eT <= tmin_lo * Alo * 0.99999905f) return false;          // t <= tMin  (factor 1 - 2^-20)
  if (Ta - eT >= c_hi * Ahi * 1.00000095f) return false;             // t >= closest (c_hi may be inf)
  return true;
}

// Three-way Moller-Trumbore decision against the reference's binary64 test
// (src/math/ray.ts:22-45) with tMin and the running closest c in [c_lo, c_hi]:
//   kTriReject  the reference certainly rejects,
//   kTriAccept  the reference certainly accepts; [t_lo, t_hi] bounds its t,
//   kTriExact   undecided: recompute in binary64,
//   kTriNearC   every condition certain but t < c: the reference accepts the
//               triangle iff its binary64 t is below c; [t_lo, t_hi] bounds t.
// Numerator bounds as in mt_candidate (2^-19 x absolute-value evaluation).
enum TriClass { kTriReject = 0, kTriAccept = 1, kTriExact = 2, kTriNearC = 3 };

LUCENT_DEV TriClass mt_classify(const Ray32& r, float4 a, float4 b, float4 c3, float tmin_lo, float tmin_hi,
                                float c_lo, float c_hi, float& t_lo, float& t_hi, float3& est) {
  const float3 e1 = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
  const float3 e2 = make_float3(c3.x - a.x, c3.y - a.y, c3.z - a.z);
  const float3 d = r.d;
  const float3 p = make_float3(d.y * e2.z - d.z * e2.y, d.z * e2.x - d.x * e2.z, d.x * e2.y - d.y * e2.x);
  const float det = e1.x * p.x + e1.y * p.y + e1.z * p.z;
  const float3 s = make_float3(r.o.x - a.x, r.o.y - a.y, r.o.z - a.z);
  const float U = s.x * p.x + s.y * p.y + s.z * p.z;
  const float3 q = make_float3(s.y * e1.z - s.z * e1.y, s.z * e1.x - s.x * e1.z, s.x * e1.y - s.y * e1.x);
  const float V = d.x * q.x + d.y * q.y + d.z * q.z;
  const float T = e2.x * q.x + e2.y * q.y + e2.z * q.z;
  const float3 ad = make_float3(fabsf(d.x), fabsf(d.y), fabsf(d.z));
  const float3 ae1 = make_float3(fabsf(e1.x), fabsf(e1.y), fabsf(e1.z));
  const float3 ae2 = make_float3(fabsf(e2.x), fabsf(e2.y), fabsf(e2.z));
  const float3 as = make_float3(fabsf(s.x), fabsf(s.y), fabsf(s.z));
  const float3 ap = make_float3(ad.y * ae2.z + ad.z * ae2.y, ad.z * ae2.x + ad.x * ae2.z, ad.x * ae2.y + ad.y * ae2.x);
  const float3 aq = make_float3(as.y * ae1.z + as.z * ae1.y, as.z * ae1.x + as.x * ae1.z, as.x * ae1.y + as.y * ae1.x);
  const float eD = fmaf(ae1.x * ap.x + ae1.y * ap.y + ae1.z * ap.z, kMtRel, kAbsFloor);
  const float eU = fmaf(as.x * ap.x + as.y * ap.y + as.z * ap.z, kMtRel, kAbsFloor);
  const float eV = fmaf(ad.x * aq.x + ad.y * aq.y + ad.z * aq.z, kMtRel, kAbsFloor);
  const float eT = fmaf(ae2.x * aq.x + ae2.y * aq.y + ae2.z * aq.z, kMtRel, kAbsFloor);

  const float A = fabsf(det);
  if (A + eD < 9.9e-13f) return kTriReject;  // |det| < 1e-12 for sure
  if (A <= eD) return kTriExact;
  const float sg = det < 0.f ? -1.f : 1.f;
  const float Ua = U * sg, Va = V * sg, Ta = T * sg;
  const float Ahi = __fadd_ru(A, eD), Alo = __fsub_rd(A, eD);
  if (Ua + eU < 0.f || Ua - eU > Ahi || Va + eV < 0.f || Ua + Va - (eU + eV) > Ahi) return kTriReject;
  if (Ta + eT < 0.f || Ta + eT <= tmin_lo * Alo * 0.99999905f) return kTriReject;  // t <= tMin
  if (Ta - eT >= c_hi * Ahi * 1.00000095f) return kTriReject;                       // t >= closest
  // Certain acceptance: every reference condition holds with margin.
  const bool inside = Ua - eU >= 0.f && Va - eV >= 0.f && Ua + Va + (eU + eV) <= Alo && Alo >= 1.0000001e-12f;
  if (!(inside && Ta - eT > tmin_hi * Ahi * 1.00000095f)) return kTriExact;
  // t = T/det lies in [(Ta-eT)/Ahi, (Ta+eT)/Alo]; round outward and widen by
  // one more ulp for the reference's own binary64 rounding.
  t_lo = __fmul_rd(__fdiv_rd(__fsub_rd(Ta, eT), Ahi), 0.99999994f);
  t_hi = __fmul_ru(__fdiv_ru(__fadd_ru(Ta, eT), Alo), 1.00000012f);
  if (!(Ta + eT < c_lo * Alo * 0.99999905f)) return kTriNearC;
  // Binary32 estimates of (t, u, v), as the GLSL's own hitTriangle computes them.
  const float inv = 1.f / det;
  est = make_float3(T * inv, U * inv, V * inv);
  return kTriAccept;
}

// ---------------------------------------------------------------------------
// The hit's t, u, v as the reference reports them (binary64, ray.ts:30-44),
// rounded to binary32, without binary64 arithmetic in the common case.
//
// Double-float values are pairs (hi, lo) of binary32 numbers with
// hi = RN(hi + lo), about 48 significant bits, built from error-free
// transformations (Knuth's TwoSum, Dekker's product through an FMA; Dekker
// 1971, "A floating-point technique for extending the available precision").
// Each double-float operation here errs by at most about 3 u^2 (u = 2^-24)
// of its operands' magnitudes, so with exact differences e1, e2, s the
// numerators U, V, T and det err by at most about 2^-44.5 x their
// absolute-value evaluations (uA, vA, tA, dA below), and a quotient x = X/det
// by 2^-44.5 (xA + |x| dA)/|det| plus 2^-46 |x|. Binary64's own rounding is
// 2^-7 of that. The bound used is 2^-42 (xA + |x| dA)/|det|, 4x the estimate,
// doubled for the binary32 rounding of the bound's own evaluation. When that
// interval around a value cannot contain a binary32 rounding boundary, the
// value's binary32 rounding equals the binary64 result's rounding; otherwise
// the caller falls back to binary64.
// ---------------------------------------------------------------------------
struct DF {
  float hi, lo;
};
LUCENT_DEV DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
LUCENT_DEV DF df_fast(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
LUCENT_DEV DF df_add(DF x, DF y) {
  DF s = df_two_sum(x.hi, y.hi);
  const DF t = df_two_sum(x.lo, y.lo);
  s = df_fast(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast(s.hi, __fadd_rn(s.lo, t.lo));
}
LUCENT_DEV DF df_sub(DF x, DF y) { return df_add(x, {-y.hi, -y.lo}); }
LUCENT_DEV DF df_mul(DF x, DF y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return df_fast(p, e);
}
LUCENT_DEV DF df_mul_f(DF x, float b) {
  const float p = __fmul_rn(x.hi, b);
  return df_fast(p, __fmaf_rn(x.lo, b, __fmaf_rn(x.hi, b, -p)));
}
LUCENT_DEV DF df_div(DF x, DF y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  DF r = df_sub(x, df_mul_f(y, q1));
  const float q2 = __fdiv_rn(r.hi, y.hi);
  r = df_sub(r, df_mul_f(y, q2));
  const float q3 = __fdiv_rn(r.hi, y.hi);
  return df_add(df_fast(q1, q2), {q3, 0.f});
}
LUCENT_DEV DF df_dot(DF ax, DF ay, DF az, DF bx, DF by, DF bz) {
  return df_add(df_add(df_mul(ax, bx), df_mul(ay, by)), df_mul(az, bz));
}

// True when every real number within `bound` of x.hi + x.lo rounds to x.hi in
// binary32 (round to nearest even). Zero, subnormal-range and tie cases say no.
LUCENT_DEV bool df_rounds_to_hi(DF x, float bound) {
  const float a = fabsf(x.hi);
  if (!(a >= 1e-30f) || !(a <= 1e30f)) return false;
  const float up = __fsub_rn(__int_as_float(__float_as_int(a) + 1), a);
  const float dn = __fsub_rn(a, __int_as_float(__float_as_int(a) - 1));
  return __fadd_ru(fabsf(x.lo), bound) < 0.5f * fminf(up, dn);
}

// The hit's (t, u, v) rounded to binary32. t always equals the rounding of
// the reference's binary64 t when this returns true; u and v are proven equal
// to theirs too when `exact_uv`, and are otherwise the roundings of the
// double-float values (at most one binary32 ulp from binary64's, and equal to
// them in all but about one case in 10^2 to 10^3, the rest being within the
// bound of a rounding boundary). False when the bound cannot prove what was
// asked.
static __device__ __noinline__ bool tri_df32(float3 o, float3 d, float4 a, float4 b, float4 c, bool exact_uv,
                                             float3& out) {
  const DF e1x = df_two_sum(b.x, -a.x), e1y = df_two_sum(b.y, -a.y), e1z = df_two_sum(b.z, -a.z);
  const DF e2x = df_two_sum(c.x, -a.x), e2y = df_two_sum(c.y, -a.y), e2z = df_two_sum(c.z, -a.z);
  const DF sx = df_two_sum(o.x, -a.x), sy = df_two_sum(o.y, -a.y), sz = df_two_sum(o.z, -a.z);
  const DF px = df_sub(df_mul_f(e2z, d.y), df_mul_f(e2y, d.z));  // p = d x e2
  const DF py = df_sub(df_mul_f(e2x, d.z), df_mul_f(e2z, d.x));
  const DF pz = df_sub(df_mul_f(e2y, d.x), df_mul_f(e2x, d.y));
  const DF det = df_dot(e1x, e1y, e1z, px, py, pz);
  const DF qx = df_sub(df_mul(sy, e1z), df_mul(sz, e1y));  // q = s x e1
  const DF qy = df_sub(df_mul(sz, e1x), df_mul(sx, e1z));
  const DF qz = df_sub(df_mul(sx, e1y), df_mul(sy, e1x));
  const DF U = df_dot(sx, sy, sz, px, py, pz);
  const DF V = df_dot({d.x, 0.f}, {d.y, 0.f}, {d.z, 0.f}, qx, qy, qz);
  const DF T = df_dot(e2x, e2y, e2z, qx, qy, qz);
  const DF t = df_div(T, det), u = df_div(U, det), v = df_div(V, det);
  // Absolute-value evaluations (binary32 is ample for a bound).
  const float3 ad = make_float3(fabsf(d.x), fabsf(d.y), fabsf(d.z));
  const float3 ae1 = make_float3(fabsf(e1x.hi), fabsf(e1y.hi), fabsf(e1z.hi));
  const float3 ae2 = make_float3(fabsf(e2x.hi), fabsf(e2y.hi), fabsf(e2z.hi));
  const float3 as = make_float3(fabsf(sx.hi), fabsf(sy.hi), fabsf(sz.hi));
  const float3 ap = make_float3(ad.y * ae2.z + ad.z * ae2.y, ad.z * ae2.x + ad.x * ae2.z, ad.x * ae2.y + ad.y * ae2.x);
  const float3 aq = make_float3(as.y * ae1.z + as.z * ae1.y, as.z * ae1.x + as.x * ae1.z, as.x * ae1.y + as.y * ae1.x);
  const float dA = ae1.x * ap.x + ae1.y * ap.y + ae1.z * ap.z;
  const float uA = as.x * ap.x + as.y * ap.y + as.z * ap.z;
  const float vA = ad.x * aq.x + ad.y * aq.y + ad.z * aq.z;
  const float tA = ae2.x * aq.x + ae2.y * aq.y + ae2.z * aq.z;
  const float g = 4.54747351e-13f / fabsf(det.hi);  // 2^-41: 2^-42 x 2 for the binary32 rounding of this bound
  if (!(g < 1e30f)) return false;
  const bool ok = df_rounds_to_hi(t, g * (tA + fabsf(t.hi) * dA)) &&
                  (!exact_uv || (df_rounds_to_hi(u, g * (uA + fabsf(u.hi) * dA)) &&
                                 df_rounds_to_hi(v, g * (vA + fabsf(v.hi) * dA))));
  out = make_float3(t.hi, u.hi, v.hi);
  return ok;
}

}  // namespace lucent
