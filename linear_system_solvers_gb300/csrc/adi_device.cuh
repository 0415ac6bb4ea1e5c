// adi_device.cuh -- device-side building blocks of the ADI time step.
//
// The arithmetic policy `X` selects between
//   X = true : every +,-,*,/ is an explicitly rounded IEEE operation (__dadd_rn, ...), so
//              the compiler cannot fuse a*b+c, and each expression keeps the reference's
//              left-to-right order -> results bit-identical to the reference's host code;
//   X = false: plain operators, the compiler contracts into FMA (rounding-level changes).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace lss_gb300 {

template <bool X> struct ar;
template <> struct ar<true> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <> struct ar<false> {
    template <typename T> static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
    template <typename T> static __device__ __forceinline__ T add(T a, T b) { return a + b; }
    template <typename T> static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
    template <typename T> static __device__ __forceinline__ T div(T a, T b) { return a / b; }
};

// Device view of one instance's time-invariant data (all arrays row-major, i*ny + j).
template <typename T> struct dev_instance {
    int nx, ny;
    T theta, zeta, gamma, delta, ni, rho, h1;
    const T *M, *P, *Z, *Mt, *Pt, *W, *C; // nx*ny each
    const T *D0, *E0, *F0;                 // nx each: D, E, F on the v = v_lo line
    const T *s_lo, *s_hi_neu, *v_hi;       // ny, ny, nx
    const int *imap, *jmap;                // nx, ny
    int ds;                                // 1: double-sweep line solves, 0: Thomas LU
};

// Stage selectors of the S-direction sweeps.
enum s_stage : int {
    S_STAGE1 = 1,    // rhs_intermed_1: explicit 9-point operator (all schemes)
    S_STAGE3_CS = 3, // Craig-Sneyd rhs_intermed_3
    S_STAGE3_MCS = 4,// modified Craig-Sneyd rhs_intermed_3
    S_STAGE4_HV = 5  // Hundsdorfer-Verwer rhs_intermed_4
};

// Right-hand side of an S-line at row t of line j, reference operation order.
//   S_STAGE1    : A = U
//   S_STAGE3_*  : A = U, B = Y1, Cc = Y2
//   S_STAGE4_HV : A = Y2, B = Y3
template <typename T, bool X, int STAGE>
__device__ __forceinline__ T s_rhs(const dev_instance<T> &d, int t, int j, const T *A, const T *B, const T *Cc,
                                    T a_low, T theta_z, T theta_p)
{
    using R = ar<X>;
    const int ny = d.ny;
    const int o = t * ny + j;
    const T one = T(1);
    if constexpr (STAGE == S_STAGE1) {
        // lss_heat_douglas_rachford_method.hpp:56-67
        const T gC = R::mul(d.gamma, d.C[o]);
        const T omt = R::sub(one, d.theta);
        const T *U = A;
        const T t1 = R::mul(gC, U[o - ny - 1]);
        const T t2 = R::mul(R::mul(omt, d.M[o]), U[o - ny]);
        const T t3 = R::mul(gC, U[o - ny + 1]);
        const T t4 = R::mul(d.Mt[o], U[o - 1]);
        const T t5 = R::mul(R::sub(R::sub(one, d.W[o]), R::mul(omt, d.Z[o])), U[o]);
        const T t6 = R::mul(d.Pt[o], U[o + 1]);
        const T t7 = R::mul(gC, U[o + ny - 1]);
        const T t8 = R::mul(R::mul(omt, d.P[o]), U[o + ny]);
        const T t9 = R::mul(gC, U[o + ny + 1]);
        return R::add(R::add(R::sub(R::add(R::add(R::add(R::sub(R::add(t1, t2), t3), t4), t5), t6), t7), t8), t9);
    } else if constexpr (STAGE == S_STAGE3_CS || STAGE == S_STAGE3_MCS) {
        // lss_heat_craig_sneyd_method.hpp:144-155; lss_heat_modified_craig_sneyd_method.hpp:147-164
        const T *U = A, *Y1 = B, *Y2 = Cc;
        T s = R::add(R::sub(R::add(R::mul(a_low, U[o - ny]), R::mul(theta_z, U[o])), R::mul(theta_p, U[o + ny])), Y1[o]);
        const T d1 = R::sub(Y2[o + ny + 1], U[o + ny + 1]);
        const T d2 = R::sub(Y2[o + ny - 1], U[o + ny - 1]);
        const T d3 = R::sub(Y2[o - ny + 1], U[o - ny + 1]);
        const T d4 = R::sub(Y2[o - ny - 1], U[o - ny - 1]);
        const T mix = R::add(R::sub(R::sub(d1, d2), d3), d4);
        s = R::add(s, R::mul(R::mul(R::mul(d.zeta, d.gamma), d.C[o]), mix));
        if constexpr (STAGE == S_STAGE3_MCS) {
            const T e1 = R::mul(d.M[o], R::sub(Y2[o - ny], U[o - ny]));
            const T e2 = R::mul(R::add(d.Z[o], d.W[o]), R::sub(Y2[o], U[o]));
            const T e3 = R::mul(d.P[o], R::sub(Y2[o + ny], U[o + ny]));
            const T e4 = R::mul(d.Mt[o], R::sub(Y2[o - 1], U[o - 1]));
            const T e5 = R::mul(d.Pt[o], R::sub(Y2[o + 1], U[o + 1]));
            s = R::add(s, R::mul(R::sub(d.zeta, d.theta), R::add(R::add(R::sub(R::sub(e1, e2), e3), e4), e5)));
        }
        return s;
    } else {
        // lss_heat_hundsdorfer_verwer_method.hpp:187-193
        const T *Y2 = A, *Y3 = B;
        return R::add(R::sub(R::add(R::mul(a_low, Y2[o - ny]), R::mul(theta_z, Y2[o])), R::mul(theta_p, Y2[o + ny])),
                      Y3[o]);
    }
}

} // namespace lss_gb300
