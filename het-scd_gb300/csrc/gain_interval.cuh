// FP32 interval enclosure of the FP64 gain model (gain.cuh).
//
// Every FP64 operation of wcc_gain has an interval counterpart with outward
// (directed) rounding in FP32.  Induction over the operations shows that the
// FP64 value wcc_gain returns lies inside the returned interval: each FP64
// result is the round-to-nearest of an exact operation on FP64 operands that
// lie in the operand intervals, the exact result lies in the outward-rounded
// FP32 interval, and rounding is monotone with FP32 bounds representable in
// FP64.  Where the model branches on a sign the interval cannot decide (a
// denominator interval containing 0, an undecidable '> 0'), or a bound is NaN,
// the result is flagged and the candidate is evaluated exactly.
//
// Use: a candidate label whose upper bound is below the best lower bound (or
// not above 0) cannot be the arg-max of the exact gains, so only the few
// surviving candidates pay for the FP64 model (FP64 runs at 1/69 of the FP32
// rate on GB300, and FP64 division at 58 Gop/s).
#pragma once

#include "gain.cuh"

namespace scd {

struct Iv {
    float lo, hi;
};

__device__ __forceinline__ Iv iv_int(int k) { return {__int2float_rd(k), __int2float_ru(k)}; }
__device__ __forceinline__ Iv iv_of(double x) { return {__double2float_rd(x), __double2float_ru(x)}; }
__device__ __forceinline__ Iv iv_add(Iv a, Iv b) { return {__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)}; }
__device__ __forceinline__ Iv iv_sub(Iv a, Iv b) { return {__fsub_rd(a.lo, b.hi), __fsub_ru(a.hi, b.lo)}; }
__device__ __forceinline__ Iv iv_neg(Iv a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ Iv iv_mul(Iv a, Iv b) {
    if (a.lo >= 0.f && b.lo >= 0.f) return {__fmul_rd(a.lo, b.lo), __fmul_ru(a.hi, b.hi)};
    const float l1 = __fmul_rd(a.lo, b.lo), l2 = __fmul_rd(a.lo, b.hi), l3 = __fmul_rd(a.hi, b.lo),
                l4 = __fmul_rd(a.hi, b.hi);
    const float h1 = __fmul_ru(a.lo, b.lo), h2 = __fmul_ru(a.lo, b.hi), h3 = __fmul_ru(a.hi, b.lo),
                h4 = __fmul_ru(a.hi, b.hi);
    return {fminf(fminf(l1, l2), fminf(l3, l4)), fmaxf(fmaxf(h1, h2), fmaxf(h3, h4))};
}

// x moved by k ulps towards -inf / +inf (finite, nonzero x)
__device__ __forceinline__ float ulps_down(float x, unsigned k) {
    const unsigned u = __float_as_uint(x);
    return __uint_as_float(x > 0.f ? u - k : u + k);
}
__device__ __forceinline__ float ulps_up(float x, unsigned k) {
    const unsigned u = __float_as_uint(x);
    return __uint_as_float(x > 0.f ? u + k : u - k);
}

// approximate reciprocal (rcp.approx.f32: at most 1 ulp from 1/x)
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// a / b for b not containing 0 (the caller checks): a * [1/b.hi, 1/b.lo], each
// reciprocal from the approximate one widened by 2 ulps; a reciprocal that is
// not a finite nonzero float marks the interval unusable
__device__ __forceinline__ Iv iv_div(Iv a, Iv b, bool *bad) {
    const float r0 = rcp_approx(b.hi), r1 = rcp_approx(b.lo);
    const float lim = 1e37f;   // keeps the 2-ulp moves inside the finite range
    if (!(fabsf(r0) < lim && fabsf(r1) < lim && r0 != 0.f && r1 != 0.f)) {
        *bad = true;
        return {0.f, 0.f};
    }
    return iv_mul(a, Iv{ulps_down(r0, 2), ulps_up(r1, 2)});
}

// 1: certainly > 0, -1: certainly < 0, 0: certainly == 0, 2: undecided
__device__ __forceinline__ int iv_sign(Iv a) {
    if (a.lo > 0.f) return 1;
    if (a.hi < 0.f) return -1;
    if (a.lo == 0.f && a.hi == 0.f) return 0;
    return 2;
}

// Interval of wcc_gain(r, d_in, d_out, c_out, p_in, p_ext, alpha); *exact_needed
// is set when the interval cannot stand in for the FP64 value.
__device__ __forceinline__ Iv wcc_gain_iv(int r, int d_in, int d_out, int c_out, Iv p_in, Iv p_ext, Iv alpha,
                                          bool *exact_needed) {
    bool bad = false;
    const Iv dr = iv_int(r);
    const Iv zero = {0.f, 0.f}, one = {1.f, 1.f};
    const Iv t = r > 0 ? iv_div(iv_int(c_out - d_in), dr, &bad) : zero;

    const Iv din_pin = iv_mul(iv_int(imul_wrap(d_in, d_in - 1)), p_in);
    Iv den = iv_add(iv_add(din_pin, iv_mul(iv_int(imul_wrap(d_out, d_out - 1)), p_ext)),
                    iv_mul(iv_int(imul_wrap(d_out, d_in)), p_ext));
    den = iv_mul(den, iv_add(iv_int(d_in + d_out), iv_mul(alpha, iv_int(r - 1 - d_in))));
    Iv A = zero;
    int sg = iv_sign(den);
    if (sg == 2) bad = true;
    else if (sg != 0) A = iv_div(iv_mul(din_pin, iv_int(d_in + d_out)), den, &bad);

    const Iv rr = iv_mul(iv_mul(iv_mul(iv_int(imul_wrap(r - 1, r - 2)), p_in), p_in), p_in);
    const Iv q = iv_mul(iv_int(r - 1), p_in);
    const Iv tr_pe = iv_mul(iv_mul(iv_mul(t, iv_int(r - 1)), p_in), p_ext);
    const Iv tt_pe = iv_mul(iv_mul(t, iv_sub(t, one)), p_ext);
    const Iv r_q = iv_sub(dr, q);

    const Iv two_din = iv_mul(iv_int(2 * (d_in - 1)), p_in);
    den = iv_add(iv_add(iv_add(iv_add(rr, two_din), tr_pe), tt_pe), iv_mul(iv_int(d_out), p_ext));
    const Iv q1t = iv_add(iv_add(q, one), t);
    den = iv_mul(den, iv_add(q1t, iv_mul(alpha, iv_sub(r_q, one))));
    Iv B = zero;
    sg = iv_sign(den);
    if (sg == 2) bad = true;
    else if (sg != 0) B = iv_div(iv_mul(two_din, q1t), den, &bad);

    den = iv_add(iv_add(rr, tt_pe), tr_pe);
    const Iv qt = iv_add(q, t);
    den = iv_mul(den, iv_add(qt, iv_mul(alpha, r_q)));
    den = iv_mul(den, iv_add(qt, iv_mul(alpha, iv_sub(r_q, one))));
    Iv C = zero;
    sg = iv_sign(den);
    const int s1 = iv_sign(iv_add(dr, t)), s2 = iv_sign(iv_add(iv_int(r - 1), t));
    if (sg == 2) bad = true;
    else if (sg != 0) {
        // C is set only if r + t > 0 and r - 1 + t > 0 (decided, or fall back)
        const bool d1 = s1 == 1, d2 = s2 == 1;
        const bool u1 = s1 == 2, u2 = s2 == 2;
        if (u1 || u2) bad = true;
        else if (d1 && d2) C = iv_div(iv_mul(iv_mul(iv_neg(rr), qt), alpha), den, &bad);
    }
    const Iv g = iv_add(iv_add(A, iv_mul(iv_int(d_in), B)), iv_mul(iv_int(r - d_in), C));
    if (!(g.lo <= g.hi)) bad = true;   // NaN bounds
    *exact_needed = bad;
    return g;
}

}  // namespace scd
