// The WCC move-gain model of the reference (src/scd.cpp:173-219; GPU twin
// src/kernels.cuh:41-92), evaluated operation by operation in IEEE double with
// explicit round-to-nearest intrinsics so that no multiply-add is contracted:
// every sum, product and quotient is rounded exactly where the reference's
// C++ (built with -ffp-contract=off) rounds it.  Integer products are int32
// with two's-complement wrap-around, as in the reference before promotion to
// double.  Kept in FP64 end to end (the reference GPU path rounds the gains to
// float, src/kernels.cuh:156-159; the CPU path, which is the parity target,
// keeps double).
#pragma once

#include <cuda_runtime.h>

namespace scd {

__device__ __forceinline__ int imul_wrap(int a, int b) { return (int)((unsigned)a * (unsigned)b); }

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double wcc_gain(int r, int d_in, int d_out, int c_out, double p_in, double p_ext,
                                        double alpha) {
    const double dr = (double)r;
    const double t = r > 0 ? ddiv((double)(c_out - d_in), dr) : 0.0;

    // A: the vertex itself
    const double din_pin = dmul((double)imul_wrap(d_in, d_in - 1), p_in);
    double den = dadd(dadd(din_pin, dmul((double)imul_wrap(d_out, d_out - 1), p_ext)),
                      dmul((double)imul_wrap(d_out, d_in), p_ext));
    den = dmul(den, dadd((double)(d_in + d_out), dmul(alpha, (double)(r - 1 - d_in))));
    double A = 0.0;
    if (den != 0.0) A = ddiv(dmul(din_pin, (double)(d_in + d_out)), den);

    // common subexpressions (identical operations in the reference, computed once)
    const double rr = dmul(dmul(dmul((double)imul_wrap(r - 1, r - 2), p_in), p_in), p_in);
    const double q = dmul((double)(r - 1), p_in);
    const double tr_pe = dmul(dmul(dmul(t, (double)(r - 1)), p_in), p_ext);   // t*(r-1)*p_in*p_ext
    const double tt_pe = dmul(dmul(t, dsub(t, 1.0)), p_ext);                  // t*(t-1)*p_ext
    const double r_q = dsub(dr, q);                                           // r - (r-1)*p_in

    // B-: neighbours inside the community
    const double two_din = dmul((double)(2 * (d_in - 1)), p_in);
    den = dadd(dadd(dadd(dadd(rr, two_din), tr_pe), tt_pe), dmul((double)d_out, p_ext));
    const double q1t = dadd(dadd(q, 1.0), t);
    den = dmul(den, dadd(q1t, dmul(alpha, dsub(r_q, 1.0))));
    double B = 0.0;
    if (den != 0.0) B = ddiv(dmul(two_din, q1t), den);

    // C-: community members not adjacent to the vertex
    den = dadd(dadd(rr, tt_pe), tr_pe);
    const double qt = dadd(q, t);
    den = dmul(den, dadd(qt, dmul(alpha, r_q)));
    den = dmul(den, dadd(qt, dmul(alpha, dsub(r_q, 1.0))));
    double C = 0.0;
    if (den != 0.0 && dadd(dr, t) > 0 && dadd((double)(r - 1), t) > 0)
        C = ddiv(dmul(dmul(-rr, qt), alpha), den);

    return dadd(dadd(A, dmul((double)d_in, B)), dmul((double)(r - d_in), C));
}

// p_int of a community as improve_partition computes it (src/scd.cpp:293-298)
__device__ __forceinline__ double community_p_in(int size, int int_edges_half) {
    if (size > 1) return ddiv(dmul(2.0, (double)int_edges_half), dmul((double)size, dsub((double)size, 1.0)));
    return 0.0;
}

}  // namespace scd
