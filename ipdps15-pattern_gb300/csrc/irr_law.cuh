// irr_law.cuh -- the built-in per-edge user functions, evaluated in FP32.
//
// The reference's user functions (moldyn/irregular.h:26-107 `map`,
// miniMD/irregular.h:109-163 `map1`) compute, for an edge (i, j),
//   d = x_i - x_j            (moldyn: minimum image, irregular.h:51-60)
//   rd = |d|^2; if rd < cutoff^2:
//   s = rd^-7 - rd^-4 / 2    (moldyn: rrd7 - 0.5*rrd4; miniMD: rrd3*(rrd3-0.5)*rrd)
//   insert(i, +d*s); insert(j, -d*s)
// in double and store the contribution as float3.  Here the per-edge
// arithmetic runs in FP32 with three safeguards so the FP32 result tracks the
// reference's:
//   * the minimum image never rounds the large |x_i - x_j| of a wrapped pair:
//     the operand above the half box is shifted first (exact by Sterbenz's
//     lemma), and the box side is carried as a float pair hi + lo so that a
//     side that is not a float (moldyn's side = (N/0.83134)^(1/3)) is not
//     rounded either;
//   * pairs whose FP32 rd falls within 2^-18 (relative) of the cutoff take
//     the reference's exact FP64 decision, so the set of contributing edges
//     is the reference's;
//   * 1/rd comes from the hardware reciprocal refined by one Newton-Raphson
//     step (r <- r + r*(1 - rd*r)), leaving it within an ulp.
// The law is antisymmetric bit for bit: f(j, i) == -f(i, j) in FP32, because
// IEEE subtraction, the wrap above and the squares are sign symmetric.  The
// owner-computes kernel relies on this to apply each edge from both ends.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace irr {

struct LawParams {
    float rc2;      // float nearest the reference's double cutoff^2
    float rc2_lo;   // rd <= rc2_lo: certainly inside
    float rc2_hi;   // rd >= rc2_hi: certainly outside
    float half;     // float(side / 2): the wrap threshold
    float side_hi;  // side = side_hi + side_lo
    float side_lo;
    int periodic;
    float half2;    // (side/2)^2 less a margin: rd <= half2 needs no wrap
    float band;     // |rd - rc2| < band: FP64 decision (rc2_lo/rc2_hi in one test)
    int pad_;
    double rc2d;    // the reference's cutoff^2 (moldyn: cutoffRadius*cutoffRadius)
    double side;
    double halfd;   // 0.5 * side, as moldyn/irregular.h:36 forms it
};

// One minimum-image component for a pair that crossed the half box.
__device__ __forceinline__ float wrap_component(float a, float b, float d0, const LawParams& P)
{
    if (d0 > P.half) return __fsub_rn(__fsub_rn(__fsub_rn(a, P.side_hi), b), P.side_lo);
    if (d0 < -P.half) return __fadd_rn(__fsub_rn(a, __fsub_rn(b, P.side_hi)), P.side_lo);
    return d0;
}

// The reference's own FP64 in/out decision for a pair at the cutoff:
// moldyn/irregular.h:47-64 with the positions widened exactly to double.
template <bool PERIODIC>
__device__ __noinline__ bool exact_inside(float4 a, float4 b, const LawParams& P)
{
    double xx = __dsub_rn((double)a.x, (double)b.x);
    double yy = __dsub_rn((double)a.y, (double)b.y);
    double zz = __dsub_rn((double)a.z, (double)b.z);
    if (PERIODIC) {
        if (xx < -P.halfd) xx = __dadd_rn(xx, P.side);
        if (yy < -P.halfd) yy = __dadd_rn(yy, P.side);
        if (zz < -P.halfd) zz = __dadd_rn(zz, P.side);
        if (xx > P.halfd) xx = __dsub_rn(xx, P.side);
        if (yy > P.halfd) yy = __dsub_rn(yy, P.side);
        if (zz > P.halfd) zz = __dsub_rn(zz, P.side);
    }
    double rd = __dadd_rn(__dadd_rn(__dmul_rn(xx, xx), __dmul_rn(yy, yy)), __dmul_rn(zz, zz));
    return rd < P.rc2d;
}

// 1/x: hardware approximation plus one Newton-Raphson step for f(r) = 1/r - x.
__device__ __forceinline__ float recip_newton(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    float e = fmaf(-x, r, 1.0f);
    return fmaf(r, e, r);
}

// Separation d = a - b (minimum image when PERIODIC) and the law's scalar s
// (force on a is d * s; 0 outside the cutoff).
template <bool PERIODIC>
__device__ __forceinline__ float lj_scalar(float4 a, float4 b, const LawParams& P, float& dx,
                                           float& dy, float& dz)
{
    dx = __fsub_rn(a.x, b.x);
    dy = __fsub_rn(a.y, b.y);
    dz = __fsub_rn(a.z, b.z);
    if (PERIODIC) {
        if (fabsf(dx) > P.half || fabsf(dy) > P.half || fabsf(dz) > P.half) {
            dx = wrap_component(a.x, b.x, dx, P);
            dy = wrap_component(a.y, b.y, dy, P);
            dz = wrap_component(a.z, b.z, dz, P);
        }
    }
    float rd = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
    bool in = rd < P.rc2;
    if (rd > P.rc2_lo && rd < P.rc2_hi) in = exact_inside<PERIODIC>(a, b, P);
    float r = recip_newton(rd);        // rd^-1
    float r2 = __fmul_rn(r, r);        // rd^-2
    float s = __fmul_rn(__fmul_rn(r2, r2), fmaf(r2, r, -0.5f));  // rd^-4 (rd^-3 - 1/2)
    return in ? s : 0.0f;
}

// Error-free sum (Knuth's TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

}  // namespace irr
