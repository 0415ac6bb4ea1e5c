// heat1d.cu -- batched 1-D implicit heat / Black-Scholes theta scheme (include/lss_heat1d.h).
//
// Reference path (MichalSara99/linear_system_solvers):
//   heat_time_loop::run / run_with_stepping  (pde_solvers/one_dimensional/heat_type/
//                                             lss_1d_general_heat_equation_implicit_kernel.hpp:83-251)
//   heat_implicit_solver_method::solve        (.../solver_method/lss_heat_implicit_solver_method.hpp:245-262)
//     implicit_heat_scheme::rhs / rhs_source  (same file :37-176), split (:200-211)
//   thomas_lu_solver::kernel                  (sparse_solvers/tridiagonal/thomas_lu_solver/
//                                             lss_thomas_lu_solver.hpp:125-191, lss_thomas_lu_boundary.hpp:114-236)
//   double_sweep_solver::kernel               (sparse_solvers/tridiagonal/double_sweep_solver/
//                                             lss_double_sweep_solver.hpp:112-155, lss_double_sweep_boundary.hpp:88-190)
//
// Layout.  Instances are sorted by size and cut into groups of 32 of equal n; a group's arrays
// are interleaved (element t of lane l at t*32 + l), so each load of a warp (one thread per
// instance, all walking their line in step) is one 256-byte (FP64) line.  Slots of a group's
// point block (n*32 elements each):
//   REFERENCE: 0 A_, 1 B_, 2 D_ (scheme coefficients), 4 gamma / L, 5 sol / K, 6 U
//   FAST:      1 WB, 2 WD (right-hand-side weights of u_t, u_{t+1} scaled by the pivot reciprocal;
//              the weight of u_{t-1} is -(1-theta)/theta * M), 3 M (a_t / beta_t), 4 G (gamma_t),
//              5 KR (k / beta_t), 6 U, 7 Y (forward sweep); slot 0 keeps A_ (unused)
// Per-step boundary values (2 per step) and source rows are interleaved the same way.  The
// whole time loop of an instance runs in one thread of one launch: there is no exchange
// between instances and no per-step launch.
#include "lss_heat1d.h"

#include "adi_common.hpp"
#include "adi_device.cuh"
#include "heat1d_schedule.hpp"

#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <thread>
#include <vector>

namespace lss_gb300 {
namespace heat1d {

constexpr int LANES = 32;
constexpr int NSLOT = 8;
// Warps per CTA of the factorised sweep, one CTA per SM: 16 in FP32 (at most 128 registers per
// thread), 8 in FP64, whose 16-point rings take ~200 registers per thread (the deeper ring
// keeps more loads in flight in each warp, which is what the longest instances, running alone
// at the end of a batch, are bound by)
template <typename T> __host__ __device__ constexpr int h1_warps() { return sizeof(T) == 4 ? 16 : 8; }
// prefetch distance (points) of the forward sweep and of the back substitution.  At most 16:
// the loads past the last row stay in H1_PAD, those below row 0 in the group's block.
constexpr int H1_PF = 16;
constexpr int H1_PFB = 16;
// elements after the last group: the sweeps may load up to the prefetch distance + 1 points past a row
constexpr long long H1_PAD = (H1_PF + 2) * LANES;
enum { S_A = 0, S_B = 1, S_D = 2, S_M = 3, S_G = 4, S_K = 5, S_U = 6, S_Y = 7 };

// One instance (device).  Solver-type scalars are stored as double (exact).
struct h1lane {
    int inst;          // creation index
    int steps;         // nt - 1
    int lo_kind, hi_kind;
    int start, end;    // first / last solved row (FAST: filled by the set-up kernel)
    int has_src;
    int forward;
    int eval_i;        // value = (1 - eval_w) U[eval_i] + eval_w U[eval_i + 1]
    int pad;
    double eval_w;
    double theta, h, k; // theta, grid step 1/(n-1), time step
    double lo_lin, hi_lin; // transformed Robin linear values (constant in time)
    double bl, bh;      // FAST: coefficients of the boundary values in the first / last row
    long long init_off; // offset of the instance's initial condition (contiguous)
};

struct h1group {
    int n, lanes, steps, pad;
    long long pt;   // point block: slot s, point t, lane l at pt + (s*n + t)*32 + l
    long long bnd;  // boundary values: step s, side q (0 lower, 1 upper) at bnd + (s*2 + q)*32 + l
    long long src;  // source rows (steps + 1) x n, or -1
    long long all;  // every time level (steps + 1) x n, or -1
};

template <typename T> struct h1params {
    const h1group *groups;
    h1lane *lanes;
    int ngroups;
    T *pt;
    const T *bnd;
    const T *src;
    T *all;
    const T *init;
    double *values;
    int *status;
    const int *warp_first; // factorised sweep: the groups of warp w are
    const int *warp_group; // warp_group[warp_first[w] .. warp_first[w + 1])
    int nwarps;
};

__device__ __forceinline__ long long el(int t) { return static_cast<long long>(t) * LANES; }
__device__ __forceinline__ double h1_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float h1_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// ------------------------------------------------------------------------------------------
// Reference order (bit-identical to the reference's host policies)
// ------------------------------------------------------------------------------------------
// implicit_heat_scheme::rhs / rhs_source at row t (lss_heat_implicit_solver_method.hpp:37-176),
// `um, uc, up` the previous solution at t-1, t, t+1 and `s0, s1` the source at time and next
// time (has_src only).  Rows 0 and N are only formed for Neumann / Robin ends.
template <typename T>
__device__ __forceinline__ T ref_rhs(int t, int N, int lo_kind, int hi_kind, T A, T B, T D, T um, T uc, T up, T th,
                                     T h, T k, T lv, T ll, T hv, T hl, bool has_src, T s0, T s1)
{
    using R = ar<true>;
    const T one = T(1), two = T(2);
    const T omt = R::sub(one, th);
    T f;
    if (t == 0) {
        const T beta = R::mul(R::mul(two, h), lv);
        const T t1 = R::mul(R::mul(omt, beta), A);
        T t2;
        if (lo_kind == LSS_HEAT1D_ROBIN) {
            const T alpha = R::mul(R::mul(two, h), ll);
            t2 = R::mul(R::sub(one, R::mul(omt, R::sub(R::mul(two, B), R::mul(alpha, A)))), uc);
        } else {
            t2 = R::mul(R::sub(one, R::mul(R::mul(two, omt), B)), uc);
        }
        const T t3 = R::mul(R::mul(omt, R::add(A, D)), up);
        f = R::add(R::add(t1, t2), t3);
        if (has_src) f = R::add(R::add(f, R::mul(R::mul(th, k), s1)), R::mul(R::mul(omt, k), s0));
    } else if (t == N) {
        const T delta = R::mul(R::mul(two, h), hv);
        const T t1 = R::mul(R::mul(omt, R::add(A, D)), um);
        T t2;
        if (hi_kind == LSS_HEAT1D_ROBIN) {
            const T gamma = R::mul(R::mul(two, h), hl);
            t2 = R::mul(R::sub(one, R::mul(omt, R::add(R::mul(two, B), R::mul(gamma, D)))), uc);
        } else {
            t2 = R::mul(R::sub(one, R::mul(R::mul(two, omt), B)), uc);
        }
        const T t3 = R::mul(R::mul(omt, delta), D);
        f = R::sub(R::add(t1, t2), t3);
        if (has_src) f = R::add(R::add(f, R::mul(R::mul(th, k), s1)), R::mul(R::mul(omt, k), s0));
    } else {
        const T t1 = R::mul(R::mul(D, omt), up);
        const T t2 = R::mul(R::sub(one, R::mul(R::mul(two, B), omt)), uc);
        const T t3 = R::mul(R::mul(A, omt), um);
        f = R::add(R::add(t1, t2), t3);
        if (has_src) f = R::add(f, R::mul(k, R::add(R::mul(th, s1), R::mul(omt, s0))));
    }
    return f;
}

// split (lss_heat_implicit_solver_method.hpp:200-211)
template <typename T> __device__ __forceinline__ void ref_split(T th, T A, T B, T D, T &a, T &b, T &c)
{
    using R = ar<true>;
    a = R::mul(-th, A);
    b = R::add(T(1), R::mul(R::mul(T(2), th), B));
    c = R::mul(-th, D);
}

template <typename T, bool DS, int PF> __global__ void __launch_bounds__(128) k_h1_ref(const h1params<T> p)
{
    using R = ar<true>;
    const int g = blockIdx.x * (blockDim.x / LANES) + threadIdx.x / LANES;
    const int lane = threadIdx.x % LANES;
    if (g >= p.ngroups) return;
    const h1group G = p.groups[g];
    if (lane >= G.lanes) return;
    const h1lane L = p.lanes[static_cast<long long>(g) * LANES + lane];
    const int n = G.n, N = n - 1;
    const long long NS = static_cast<long long>(n) * LANES;
    T *base = p.pt + G.pt + lane;
    const T *A = base + S_A * NS, *B = base + S_B * NS, *D = base + S_D * NS;
    T *GM = base + S_G * NS, *SL = base + S_K * NS, *U = base + S_U * NS;
    const T *BND = p.bnd + G.bnd + lane;
    const bool has_src = L.has_src != 0;
    const T *SRC = has_src ? p.src + G.src + lane : nullptr;
    T *ALL = G.all >= 0 ? p.all + G.all + lane : nullptr;
    const T th = T(L.theta), h = T(L.h), k = T(L.k), ll = T(L.lo_lin), hl = T(L.hi_lin);
    const T two = T(2), one = T(1);
    const int lo_kind = L.lo_kind, hi_kind = L.hi_kind;
    const int steps = L.steps;

    for (int t = 0; t < n; ++t) U[el(t)] = p.init[L.init_off + t];
    int row = L.forward ? 0 : steps;
    if (ALL)
        for (int t = 0; t < n; ++t) ALL[(static_cast<long long>(row) * n + t) * LANES] = U[el(t)];

    for (int s = 0; s < steps; ++s) {
        const T lv = BND[el(2 * s)], hv = BND[el(2 * s + 1)];
        const T *S0 = has_src ? SRC + static_cast<long long>(s) * NS : nullptr;
        const T *S1 = has_src ? S0 + NS : nullptr;
        auto rhs_v = [&](int t, T Av, T Bv, T Dv, T um, T uc, T up) -> T {
            return ref_rhs<T>(t, N, lo_kind, hi_kind, Av, Bv, Dv, um, uc, up, th, h, k, lv, ll, hv, hl, has_src,
                              has_src ? S0[el(t)] : T(0), has_src ? S1[el(t)] : T(0));
        };
        auto rhs = [&](int t, T um, T uc, T up) -> T { return rhs_v(t, A[el(t)], B[el(t)], D[el(t)], um, uc, up); };
        // rings of PF points: the loads of point t + PF are issued before point t is computed
        T ra[PF], rb[PF], rd[PF], ru[PF];
        auto load_pt = [&](int j, int t) {
            ra[j] = A[el(t)];
            rb[j] = B[el(t)];
            rd[j] = D[el(t)];
            ru[j] = t < N ? U[el(t + 1)] : T(0);
        };
        if (!DS) {
            // thomas_lu_solver::kernel: init_coefficients, forward loops (fused: each value is
            // computed as in the reference's separate beta/gamma and solution loops), back substitution
            const int start = lo_kind == LSS_HEAT1D_DIRICHLET ? 1 : 0;
            const int end = hi_kind == LSS_HEAT1D_DIRICHLET ? n - 2 : n - 1;
            T um = start ? U[el(0)] : T(0), uc = U[el(start)], up = U[el(start + 1)];
            T a, b, c;
            ref_split(th, A[el(start)], B[el(start)], D[el(start)], a, b, c);
            const T f0 = rhs(start, um, uc, up);
            T beta, gam, z;
            if (lo_kind == LSS_HEAT1D_DIRICHLET) {
                beta = b;
                gam = R::div(c, beta);
                z = R::div(R::sub(f0, R::mul(a, lv)), beta);
            } else {
                const T cst = R::mul(R::mul(two, h), lv);
                beta = lo_kind == LSS_HEAT1D_ROBIN ? R::add(b, R::mul(a, R::mul(R::mul(two, h), ll))) : b;
                gam = R::div(R::add(a, c), beta);
                z = R::div(R::sub(f0, R::mul(a, cst)), beta);
            }
            GM[el(start)] = gam;
            SL[el(start)] = z;
            T sol = z;
#pragma unroll
            for (int j = 0; j < PF; ++j)
                if (start + 1 + j < end) load_pt(j, start + 1 + j);
            for (int tb = start + 1; tb < end; tb += PF) {
#pragma unroll
                for (int j = 0; j < PF; ++j) {
                    const int t = tb + j;
                    if (t < end) {
                        const T Av = ra[j], Bv = rb[j], Dv = rd[j], un = ru[j];
                        if (t + PF < end) load_pt(j, t + PF);
                        um = uc;
                        uc = up;
                        up = un;
                        ref_split(th, Av, Bv, Dv, a, b, c);
                        const T f = rhs_v(t, Av, Bv, Dv, um, uc, up);
                        beta = R::sub(b, R::mul(a, gam));
                        gam = R::div(c, beta);
                        sol = R::div(R::sub(f, R::mul(a, sol)), beta);
                        GM[el(t)] = gam;
                        SL[el(t)] = sol;
                    }
                }
            }
            // final_coefficients at the last solved row
            um = uc;
            uc = up;
            up = end < N ? U[el(end + 1)] : T(0);
            ref_split(th, A[el(end)], B[el(end)], D[el(end)], a, b, c);
            const T fe = rhs(end, um, uc, up);
            T an, bn, rn;
            if (hi_kind == LSS_HEAT1D_DIRICHLET) {
                an = a;
                bn = b;
                rn = R::sub(fe, R::mul(c, hv));
            } else {
                const T cst = R::mul(R::mul(two, h), hv);
                an = R::add(a, c);
                bn = hi_kind == LSS_HEAT1D_ROBIN ? R::sub(b, R::mul(c, R::mul(R::mul(two, h), hl))) : b;
                rn = R::add(fe, R::mul(c, cst));
            }
            const T beta_e = R::sub(bn, R::mul(an, gam));
            T x = R::div(R::sub(rn, R::mul(an, sol)), beta_e);
            U[el(end)] = x;
#pragma unroll
            for (int j = 0; j < PF; ++j)
                if (end - 1 - j >= start) {
                    ra[j] = SL[el(end - 1 - j)];
                    rb[j] = GM[el(end - 1 - j)];
                }
            for (int tb = end - 1; tb >= start; tb -= PF) {
#pragma unroll
                for (int j = 0; j < PF; ++j) {
                    const int t = tb - j;
                    if (t >= start) {
                        const T sv = ra[j], gv = rb[j];
                        if (t - PF >= start) {
                            ra[j] = SL[el(t - PF)];
                            rb[j] = GM[el(t - PF)];
                        }
                        x = R::sub(sv, R::mul(gv, x));
                        U[el(t)] = x;
                    }
                }
            }
            if (start == 1) U[el(0)] = lv;
            if (end == N - 1) U[el(N)] = hv;
        } else {
            // double_sweep_solver::kernel
            const int start = lo_kind == LSS_HEAT1D_DIRICHLET ? 1 : 0;
            const int end = hi_kind == LSS_HEAT1D_DIRICHLET ? n - 2 : n - 1;
            T Kp, Lp;
            T um = U[el(0)], uc = U[el(0)], up = U[el(1)];
            T a, b, c;
            if (lo_kind == LSS_HEAT1D_DIRICHLET) {
                Kp = lv;
                Lp = T(0);
            } else {
                ref_split(th, A[el(0)], B[el(0)], D[el(0)], a, b, c);
                const T f0 = rhs(0, T(0), uc, up);
                const T den = lo_kind == LSS_HEAT1D_ROBIN ? R::add(b, R::mul(R::mul(R::mul(a, h), two), ll)) : b;
                Kp = R::div(R::sub(f0, R::mul(R::mul(R::mul(a, h), two), lv)), den);
                Lp = R::div(R::mul(T(-1), R::add(a, c)), den);
            }
            SL[el(0)] = Kp;
            GM[el(0)] = Lp;
            T Kq = T(0), Lq = T(0); // K_{N-1}, L_{N-1} when the loop ends at N
#pragma unroll
            for (int j = 0; j < PF; ++j)
                if (1 + j <= end) load_pt(j, 1 + j);
            for (int tb = 1; tb <= end; tb += PF) {
#pragma unroll
                for (int j = 0; j < PF; ++j) {
                    const int t = tb + j;
                    if (t <= end) {
                        const T Av = ra[j], Bv = rb[j], Dv = rd[j], un = ru[j];
                        if (t + PF <= end) load_pt(j, t + PF);
                        um = uc;
                        uc = up;
                        up = un;
                        ref_split(th, Av, Bv, Dv, a, b, c);
                        const T f = rhs_v(t, Av, Bv, Dv, um, uc, up);
                        const T tmp = R::add(b, R::mul(a, Lp));
                        const T Ln = R::div(R::mul(T(-1), c), tmp);
                        const T Kn = R::div(R::sub(f, R::mul(a, Kp)), tmp);
                        Kq = Kp;
                        Lq = Lp;
                        Kp = Kn;
                        Lp = Ln;
                        SL[el(t)] = Kn;
                        GM[el(t)] = Ln;
                    }
                }
            }
            T x;
            if (hi_kind == LSS_HEAT1D_DIRICHLET) {
                x = hv;
            } else {
                // loop ended at t = N: (Kp, Lp) = (K_N, L_N), (Kq, Lq) = (K_{N-1}, L_{N-1})
                const T cst = R::mul(R::mul(two, h), hv);
                const T den = hi_kind == LSS_HEAT1D_ROBIN
                                  ? R::sub(one, R::mul(Lp, R::sub(Lq, R::mul(R::mul(two, h), hl))))
                                  : R::sub(one, R::mul(Lp, Lq));
                x = R::div(R::add(R::mul(Lp, R::sub(Kq, cst)), Kp), den);
            }
            U[el(N)] = x;
#pragma unroll
            for (int j = 0; j < PF; ++j)
                if (N - 1 - j >= start) {
                    ra[j] = SL[el(N - 1 - j)];
                    rb[j] = GM[el(N - 1 - j)];
                }
            for (int tb = N - 1; tb >= start; tb -= PF) {
#pragma unroll
                for (int j = 0; j < PF; ++j) {
                    const int t = tb - j;
                    if (t >= start) {
                        const T kv = ra[j], lv2 = rb[j];
                        if (t - PF >= start) {
                            ra[j] = SL[el(t - PF)];
                            rb[j] = GM[el(t - PF)];
                        }
                        x = R::add(R::mul(lv2, x), kv);
                        U[el(t)] = x;
                    }
                }
            }
            if (start == 1) U[el(0)] = lv;
        }
        row += L.forward ? 1 : -1;
        if (ALL)
            for (int t = 0; t < n; ++t) ALL[(static_cast<long long>(row) * n + t) * LANES] = U[el(t)];
    }
    // value at the evaluation point and finiteness of the final solution
    int bad = 0;
    for (int t = 0; t < n; ++t) bad |= !isfinite(static_cast<double>(U[el(t)]));
    const int i = L.eval_i;
    p.values[L.inst] = (1.0 - L.eval_w) * static_cast<double>(U[el(i)]) + L.eval_w * static_cast<double>(U[el(i + 1)]);
    p.status[L.inst] = bad;
}

// ------------------------------------------------------------------------------------------
// FAST: one factorisation per instance (set-up), then per step one fused right-hand-side +
// forward sweep y_t = WB u_t + WD u_{t+1} + M (kap u_{t-1} - y_{t-1}) (+ boundary / source
// terms; kap = -(1-theta)/theta) and one back substitution x_t = y_t - G x_{t+1}.  Four loads,
// one store and four FP64 operations per point forward; two loads, one store and one FMA per
// point backward: 64 bytes per point-step in FP64.
// ------------------------------------------------------------------------------------------
template <typename T> __global__ void __launch_bounds__(128) k_h1_setup_fast(const h1params<T> p)
{
    const int g = blockIdx.x * (blockDim.x / LANES) + threadIdx.x / LANES;
    const int lane = threadIdx.x % LANES;
    if (g >= p.ngroups) return;
    const h1group G = p.groups[g];
    if (lane >= G.lanes) return;
    h1lane &L = p.lanes[static_cast<long long>(g) * LANES + lane];
    const int n = G.n, N = n - 1;
    const long long NS = static_cast<long long>(n) * LANES;
    T *base = p.pt + G.pt + lane;
    T *WA = base + S_A * NS, *WB = base + S_B * NS, *WD = base + S_D * NS;
    T *M = base + S_M * NS, *GG = base + S_G * NS, *KR = base + S_K * NS;
    const T th = T(L.theta), h2 = T(2) * T(L.h), k = T(L.k), ll = T(L.lo_lin), hl = T(L.hi_lin);
    const T one = T(1), omt = one - th;
    const int start = L.lo_kind == LSS_HEAT1D_DIRICHLET ? 1 : 0;
    const int end = L.hi_kind == LSS_HEAT1D_DIRICHLET ? N - 1 : N;
    T gam = T(0), bl = T(0), bh = T(0);
    for (int t = 0; t < n; ++t) {
        const T A = WA[el(t)], B = WB[el(t)], D = WD[el(t)];
        if (t < start || t > end) {
            WB[el(t)] = WD[el(t)] = M[el(t)] = GG[el(t)] = KR[el(t)] = T(0);
            continue;
        }
        const T a = -th * A, b = one + T(2) * th * B, c = -th * D;
        T beta, wa, wb, wd, m;
        if (t == start && start == 0) { // Neumann / Robin lower row
            beta = L.lo_kind == LSS_HEAT1D_ROBIN ? b + a * (h2 * ll) : b;
            gam = (a + c) / beta;
            const T rb = one / beta;
            wa = T(0);
            wb = (L.lo_kind == LSS_HEAT1D_ROBIN ? one - omt * (T(2) * B - h2 * ll * A) : one - T(2) * omt * B) * rb;
            wd = omt * (A + D) * rb;
            m = T(0);
            bl = (omt * h2 * A - a * h2) * rb;
            KR[el(t)] = k * rb;
        } else if (t == end && end == N) { // Neumann / Robin upper row
            const T an = a + c;
            const T bn = L.hi_kind == LSS_HEAT1D_ROBIN ? b - c * (h2 * hl) : b;
            beta = bn - an * gam;
            const T rb = one / beta;
            wa = omt * (A + D) * rb;
            wb = (L.hi_kind == LSS_HEAT1D_ROBIN ? one - omt * (T(2) * B + h2 * hl * D) : one - T(2) * omt * B) * rb;
            wd = T(0);
            m = an * rb;
            bh = (c * h2 - omt * h2 * D) * rb;
            gam = T(0);
            KR[el(t)] = k * rb;
        } else { // interior row (the first one after a Dirichlet end uses y_0 = lower value)
            beta = t == start ? b : b - a * gam;
            gam = c / beta;
            const T rb = one / beta;
            wa = omt * A * rb;
            wb = (one - T(2) * omt * B) * rb;
            wd = omt * D * rb;
            m = a * rb;
            if (t == end) bh = -c * rb; // Dirichlet upper end: - c_{N-1} v_hi / beta_{N-1}
            KR[el(t)] = k * rb;
        }
        (void)wa; // = kap * m, formed by the sweep
        WB[el(t)] = wb;
        WD[el(t)] = wd;
        M[el(t)] = m;
        GG[el(t)] = gam;
    }
    L.start = start;
    L.end = end;
    L.bl = static_cast<double>(bl);
    L.bh = static_cast<double>(bh);
}

// Time loop of group g in one warp.  Per step: the first solved row, the interior rows in
// blocks of PF (the loads of point t + PF are issued before point t is computed, from a ring of
// PF registers per array; loads past the last row stay inside the group's block and are never
// used), the last solved row, then the back substitution the same way downwards.  SRC: the
// batch has heat sources; KEEP: every time level is written out.
template <typename T, int PF, bool SRC, bool KEEP>
__device__ __forceinline__ void h1_fast_group(const h1params<T> p, const int g, const int lane)
{
    const h1group G = p.groups[g];
    if (lane >= G.lanes) return;
    const h1lane L = p.lanes[static_cast<long long>(g) * LANES + lane];
    const int n = G.n, N = n - 1;
    const int NS = n * LANES;
    T *base = p.pt + G.pt + lane;
    const T *__restrict__ WB = base + S_B * NS;
    const T *__restrict__ WD = base + S_D * NS;
    const T *__restrict__ M = base + S_M * NS;
    const T *__restrict__ GG = base + S_G * NS;
    const T *__restrict__ KR = base + S_K * NS;
    T *__restrict__ U = base + S_U * NS;
    T *__restrict__ Y = base + S_Y * NS;
    const T *BND = p.bnd + G.bnd + lane;
    const bool has_src = SRC && L.has_src != 0;
    const T *SRCP = has_src ? p.src + G.src + lane : nullptr;
    T *ALL = KEEP ? p.all + G.all + lane : nullptr;
    const T th = T(L.theta), omt = T(1) - th, bl = T(L.bl), bh = T(L.bh);
    const T kap = -omt / th; // -1 (Crank-Nicolson) or 0 (Euler), exact
    const bool cn = kap != T(0);
    const int start = L.start, end = L.end, steps = L.steps;
    const int S = LANES;

    for (int t = 0; t < n; ++t) U[t * S] = p.init[L.init_off + t];
    int row = L.forward ? 0 : steps;
    if (KEEP)
        for (int t = 0; t < n; ++t) ALL[(static_cast<long long>(row) * n + t) * S] = U[t * S];

    for (int s = 0; s < steps; ++s) {
        const T lv = BND[(2 * s) * S], hv = BND[(2 * s + 1) * S];
        const T *S0 = has_src ? SRCP + static_cast<long long>(s) * NS : nullptr;
        auto src_term = [&](int t) -> T {
            return has_src ? KR[t * S] * (th * S0[NS + t * S] + omt * S0[t * S]) : T(0);
        };
        // first solved row.  Every row's weight of u_{t-1} is kap * M_t (a_t = -theta A_t, so
        // (1 - theta) A_t / beta_t = kap a_t / beta_t, also in the Neumann / Robin end rows):
        // y_t = WB u_t + WD u_{t+1} + M (kap u_{t-1} - y_{t-1}), four loads per point
        T um = start ? U[0] : T(0);
        T uc = U[start * S];
        T up = U[(start + 1) * S];
        T yp = WB[start * S] * uc + WD[start * S] * up + M[start * S] * (kap * um - (start ? lv : T(0)));
        if (start == 0) yp += bl * lv;
        yp += src_term(start);
        Y[start * S] = yp;
        um = uc;
        uc = up;
        // interior rows start+1 .. end-1 as y_t = c_t - M_t y_{t-1}, c_t = WB u_t + WD u_{t+1}
        // - [CN] M_t u_{t-1} (+ source): c_t does not depend on the recurrence, so the dependent
        // chain through y is one FMA per point
        T rwb[PF], rwd[PF], rm[PF], rup[PF];
        int t = start + 1;
#pragma unroll
        for (int j = 0; j < PF; ++j) {
            const int q = (t + j) * S;
            rwb[j] = WB[q];
            rwd[j] = WD[q];
            rm[j] = M[q];
            rup[j] = U[q + S];
        }
        for (; t + PF <= end; t += PF) {
#pragma unroll
            for (int j = 0; j < PF; ++j) {
                const T wb = rwb[j], wd = rwd[j], m = rm[j], u1 = rup[j];
                const int q = (t + j + PF) * S;
                rwb[j] = WB[q];
                rwd[j] = WD[q];
                rm[j] = M[q];
                rup[j] = U[q + S];
                T c = h1_fma(-m, cn ? um : T(0), h1_fma(wd, u1, wb * uc));
                if (SRC) c += src_term(t + j);
                const T y = h1_fma(-m, yp, c);
                Y[(t + j) * S] = y;
                yp = y;
                um = uc;
                uc = u1;
            }
        }
#pragma unroll
        for (int j = 0; j < PF; ++j) {
            if (t + j < end) {
                T c = h1_fma(-rm[j], cn ? um : T(0), h1_fma(rwd[j], rup[j], rwb[j] * uc));
                if (SRC) c += src_term(t + j);
                const T y = h1_fma(-rm[j], yp, c);
                Y[(t + j) * S] = y;
                yp = y;
                um = uc;
                uc = rup[j];
            }
        }
        // last solved row
        T x = yp;
        if (end > start) {
            const int q = end * S;
            const T u1 = end < N ? U[q + S] : T(0);
            x = WB[q] * uc + WD[q] * u1 + M[q] * (kap * um - yp) + bh * hv;
            x += src_term(end);
        }
        U[end * S] = x;
        // back substitution end-1 .. start (loads down to PFB <= 16 rows below row start - 1 stay
        // inside the group's block: G and Y have at least 4n >= 16 rows of other slots below them)
        constexpr int PFB = H1_PFB;
        T ry[PFB], rg[PFB];
        t = end - 1;
#pragma unroll
        for (int j = 0; j < PFB; ++j) {
            const int q = (t - j) * S;
            ry[j] = Y[q];
            rg[j] = GG[q];
        }
        for (; t - PFB >= start - 1; t -= PFB) {
#pragma unroll
            for (int j = 0; j < PFB; ++j) {
                const T yv = ry[j], gv = rg[j];
                const int q = (t - j - PFB) * S;
                ry[j] = Y[q];
                rg[j] = GG[q];
                x = yv - gv * x;
                U[(t - j) * S] = x;
            }
        }
#pragma unroll
        for (int j = 0; j < PFB; ++j) {
            if (t - j >= start) {
                x = ry[j] - rg[j] * x;
                U[(t - j) * S] = x;
            }
        }
        if (start == 1) U[0] = lv;
        if (end == N - 1) U[N * S] = hv;
        row += L.forward ? 1 : -1;
        if (KEEP)
            for (int q = 0; q < n; ++q) ALL[(static_cast<long long>(row) * n + q) * S] = U[q * S];
    }
    int bad = 0;
    for (int q = 0; q < n; ++q) bad |= !isfinite(static_cast<double>(U[q * S]));
    const int i = L.eval_i;
    p.values[L.inst] = (1.0 - L.eval_w) * static_cast<double>(U[i * S]) + L.eval_w * static_cast<double>(U[(i + 1) * S]);
    p.status[L.inst] = bad;
}

// One CTA of h1_warps<T>() warps per SM (the register file holds one CTA); warp w runs the groups warp_group[warp_first[w] .. warp_first[w + 1]) placed by
// schedule_groups.
template <typename T, int PF, bool SRC, bool KEEP>
__global__ void __launch_bounds__(h1_warps<T>() * LANES, 1) k_h1_fast(const h1params<T> p)
{
    const int w = blockIdx.x * (blockDim.x / LANES) + threadIdx.x / LANES;
    const int lane = threadIdx.x % LANES;
    if (w >= p.nwarps) return;
    const int q1 = p.warp_first[w + 1];
    for (int q = p.warp_first[w]; q < q1; ++q) h1_fast_group<T, PF, SRC, KEEP>(p, p.warp_group[q], lane);
}

// scatter of per-instance contiguous tables into the interleaved group layout (the instance of
// a flat position found by binary search over the instances' offsets)
// coef (3 rows of n) -> slots 0..2
template <typename T>
__global__ void k_h1_scatter_coef(const h1group *groups, const int *ig, const int *il, const long long *off,
                                  const int *nn, int count, const T *flat, T *pt, long long total)
{
    for (long long q = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; q < total;
         q += static_cast<long long>(gridDim.x) * blockDim.x) {
        // locate the instance by binary search over offsets (3n elements each)
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (off[mid] <= q) lo = mid; else hi = mid - 1;
        }
        const int inst = lo;
        const long long r = q - off[inst];
        const int n = nn[inst];
        const int slot = static_cast<int>(r / n), t = static_cast<int>(r % n);
        const h1group G = groups[ig[inst]];
        pt[G.pt + (static_cast<long long>(slot) * n + t) * LANES + il[inst]] = flat[q];
    }
}

// rows x len per instance (boundary values: len 2, source: len n) -> interleaved at `field`
template <typename T>
__global__ void k_h1_scatter_rows(const h1group *groups, const int *ig, const int *il, const long long *off,
                                  const int *len, int count, const T *flat, T *dst, int field, long long total)
{
    for (long long q = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; q < total;
         q += static_cast<long long>(gridDim.x) * blockDim.x) {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (off[mid] <= q) lo = mid; else hi = mid - 1;
        }
        const int inst = lo;
        const long long r = q - off[inst];
        const h1group G = groups[ig[inst]];
        const long long base = field == 0 ? G.bnd : G.src;
        dst[base + r * LANES + il[inst]] = flat[q];
    }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
struct inst_info {
    int n, nt, lo_kind, hi_kind, has_src, forward, theta_scheme;
    double t_lo, t_hi, lo_lin, hi_lin;
    int eval_i;
    double eval_w;
};

template <typename T> struct host_tables {
    std::vector<T> coef, init, bnd, src; // coef 3n, init n, bnd 2*steps, src (steps+1)*n
    std::vector<T> x;                    // physical grid (Black-Scholes)
};

struct batch_base {
    virtual ~batch_base() = default;
    int precision = LSS_ADI_FP64, arith = LSS_ADI_ARITH_FAST, options = 0, count = 0;
    double point_steps = 0;
};

template <typename T> struct batch_t : batch_base {
    std::vector<inst_info> info;
    std::vector<h1group> groups;
    std::vector<h1lane> lanes;
    std::vector<int> inst_group, inst_lane;
    std::vector<long long> init_off;
    std::vector<std::vector<T>> grids;
    long long total_init = 0;
    dbuf<h1group> d_groups;
    dbuf<h1lane> d_lanes;
    dbuf<T> d_pt, d_bnd, d_src, d_all, d_init;
    dbuf<double> d_values;
    dbuf<int> d_status;
    warp_schedule sched;          // placement of the groups for the factorised sweep
    dbuf<int> d_wfirst, d_wgroup;
    bool ds = false;

    h1params<T> params()
    {
        h1params<T> p{};
        p.groups = d_groups.p;
        p.lanes = d_lanes.p;
        p.ngroups = static_cast<int>(groups.size());
        p.pt = d_pt.p;
        p.bnd = d_bnd.p;
        p.src = d_src.p;
        p.all = d_all.p;
        p.init = d_init.p;
        p.values = d_values.p;
        p.status = d_status.p;
        p.warp_first = d_wfirst.p;
        p.warp_group = d_wgroup.p;
        p.nwarps = sched.ctas * sched.warps_per_cta;
        return p;
    }
    int build(std::vector<inst_info> &&inf, std::vector<host_tables<T>> &tabs);
    int run(cudaStream_t s);
};

static int check_theta(int th)
{
    return th == LSS_ADI_EULER || th == LSS_ADI_CRANK_NICOLSON;
}

template <typename T> int batch_t<T>::build(std::vector<inst_info> &&inf, std::vector<host_tables<T>> &tabs)
{
    info = std::move(inf);
    count = static_cast<int>(info.size());
    // sort by size (desc), then steps (desc): equal-size groups of 32 with similar time loops
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (info[a].n != info[b].n) return info[a].n > info[b].n;
        return info[a].nt > info[b].nt;
    });
    inst_group.assign(count, 0);
    inst_lane.assign(count, 0);
    long long pt = 0, bnd = 0, src = 0, all = 0;
    const bool keep_all = (options & LSS_HEAT1D_OPT_ALL_STEPS) != 0;
    for (int q = 0; q < count;) {
        const int n = info[order[q]].n;
        h1group G{};
        G.n = n;
        int l = 0, steps = 0, gsrc = 0;
        while (q + l < count && l < LANES && info[order[q + l]].n == n) {
            steps = std::max(steps, info[order[q + l]].nt - 1);
            gsrc |= info[order[q + l]].has_src;
            ++l;
        }
        G.lanes = l;
        G.steps = steps;
        G.pt = pt;
        pt += static_cast<long long>(NSLOT) * n * LANES;
        G.bnd = bnd;
        bnd += 2LL * steps * LANES;
        G.src = gsrc ? src : -1;
        if (gsrc) src += static_cast<long long>(steps + 1) * n * LANES;
        G.all = keep_all ? all : -1;
        if (keep_all) all += static_cast<long long>(steps + 1) * n * LANES;
        const int gi = static_cast<int>(groups.size());
        for (int j = 0; j < l; ++j) {
            inst_group[order[q + j]] = gi;
            inst_lane[order[q + j]] = j;
        }
        groups.push_back(G);
        q += l;
    }
    // lanes and contiguous initial conditions
    lanes.assign(groups.size() * LANES, h1lane{});
    for (auto &L : lanes) L.inst = -1;
    init_off.assign(count, 0);
    total_init = 0;
    point_steps = 0;
    for (int i = 0; i < count; ++i) {
        init_off[i] = total_init;
        total_init += info[i].n;
        point_steps += static_cast<double>(info[i].n) * (info[i].nt - 1);
        const inst_info &f = info[i];
        h1lane &L = lanes[static_cast<size_t>(inst_group[i]) * LANES + inst_lane[i]];
        L.inst = i;
        L.steps = f.nt - 1;
        L.lo_kind = f.lo_kind;
        L.hi_kind = f.hi_kind;
        L.start = f.lo_kind == LSS_HEAT1D_DIRICHLET ? 1 : 0;
        L.end = f.hi_kind == LSS_HEAT1D_DIRICHLET ? f.n - 2 : f.n - 1;
        L.has_src = f.has_src;
        L.forward = f.forward;
        L.eval_i = f.eval_i;
        L.eval_w = f.eval_w;
        const T one = T(1.0);
        L.theta = f.theta_scheme == LSS_ADI_EULER ? 1.0 : 0.5;
        L.h = static_cast<double>(one / static_cast<T>(static_cast<size_t>(f.n - 1)));
        L.k = static_cast<double>((static_cast<T>(f.t_hi) - static_cast<T>(f.t_lo)) / static_cast<T>(static_cast<size_t>(f.nt - 1)));
        L.lo_lin = f.lo_lin;
        L.hi_lin = f.hi_lin;
        L.init_off = init_off[i];
    }
    // flat host arrays in creation order
    std::vector<T> coef_flat, init_flat(total_init), bnd_flat, src_flat;
    std::vector<long long> coef_off(count), bnd_off(count), src_off(count);
    std::vector<int> nn(count);
    long long cpos = 0, bpos = 0, spos = 0;
    for (int i = 0; i < count; ++i) {
        coef_off[i] = cpos;
        cpos += 3LL * info[i].n;
        bnd_off[i] = bpos;
        bpos += 2LL * (info[i].nt - 1);
        src_off[i] = spos;
        if (info[i].has_src) spos += static_cast<long long>(info[i].nt) * info[i].n;
        nn[i] = info[i].n;
    }
    coef_flat.resize(cpos);
    bnd_flat.resize(bpos);
    src_flat.resize(spos);
    for (int i = 0; i < count; ++i) {
        std::copy(tabs[i].coef.begin(), tabs[i].coef.end(), coef_flat.begin() + coef_off[i]);
        std::copy(tabs[i].init.begin(), tabs[i].init.end(), init_flat.begin() + init_off[i]);
        std::copy(tabs[i].bnd.begin(), tabs[i].bnd.end(), bnd_flat.begin() + bnd_off[i]);
        if (info[i].has_src) std::copy(tabs[i].src.begin(), tabs[i].src.end(), src_flat.begin() + src_off[i]);
        if (!tabs[i].x.empty()) grids.push_back(std::move(tabs[i].x));
        std::vector<T>().swap(tabs[i].coef);
        std::vector<T>().swap(tabs[i].bnd);
        std::vector<T>().swap(tabs[i].src);
    }
    LSS_CUDA_TRY(d_groups.alloc(groups.size()), "heat1d: allocating groups");
    LSS_CUDA_TRY(d_groups.upload(groups.data(), groups.size()), "heat1d: uploading groups");
    LSS_CUDA_TRY(d_lanes.alloc(lanes.size()), "heat1d: allocating lanes");
    LSS_CUDA_TRY(d_lanes.upload(lanes.data(), lanes.size()), "heat1d: uploading lanes");
    LSS_CUDA_TRY(d_pt.alloc(pt + H1_PAD), "heat1d: allocating point arrays");
    LSS_CUDA_TRY(cudaMemset(d_pt.p, 0, (pt + H1_PAD) * sizeof(T)), "heat1d: clearing point arrays");
    LSS_CUDA_TRY(d_bnd.alloc(std::max(1LL, bnd)), "heat1d: allocating boundary values");
    LSS_CUDA_TRY(cudaMemset(d_bnd.p, 0, d_bnd.n * sizeof(T)), "heat1d: clearing boundary values");
    if (src > 0) {
        LSS_CUDA_TRY(d_src.alloc(src), "heat1d: allocating source rows");
        LSS_CUDA_TRY(cudaMemset(d_src.p, 0, src * sizeof(T)), "heat1d: clearing source rows");
    }
    if (all > 0) LSS_CUDA_TRY(d_all.alloc(all), "heat1d: allocating time levels");
    LSS_CUDA_TRY(d_init.alloc(total_init), "heat1d: allocating initial conditions");
    LSS_CUDA_TRY(d_init.upload(init_flat.data(), total_init), "heat1d: uploading initial conditions");
    LSS_CUDA_TRY(d_values.alloc(count), "heat1d: allocating values");
    LSS_CUDA_TRY(d_status.alloc(count), "heat1d: allocating status");
    {
        dbuf<int> d_ig, d_il, d_nn, d_len;
        dbuf<long long> d_off;
        dbuf<T> d_flat;
        LSS_CUDA_TRY(d_ig.alloc(count), "heat1d: set-up");
        LSS_CUDA_TRY(d_ig.upload(inst_group.data(), count), "heat1d: set-up");
        LSS_CUDA_TRY(d_il.alloc(count), "heat1d: set-up");
        LSS_CUDA_TRY(d_il.upload(inst_lane.data(), count), "heat1d: set-up");
        LSS_CUDA_TRY(d_nn.alloc(count), "heat1d: set-up");
        LSS_CUDA_TRY(d_nn.upload(nn.data(), count), "heat1d: set-up");
        LSS_CUDA_TRY(d_off.alloc(count), "heat1d: set-up");
        // coefficient tables
        LSS_CUDA_TRY(d_off.upload(coef_off.data(), count), "heat1d: set-up");
        LSS_CUDA_TRY(d_flat.alloc(cpos), "heat1d: set-up");
        LSS_CUDA_TRY(d_flat.upload(coef_flat.data(), cpos), "heat1d: set-up");
        k_h1_scatter_coef<T><<<std::min(grid_for(cpos, 256), 65535), 256>>>(d_groups.p, d_ig.p, d_il.p, d_off.p,
                                                                           d_nn.p, count, d_flat.p, d_pt.p, cpos);
        LSS_CUDA_TRY(cudaGetLastError(), "heat1d: scattering coefficients");
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "heat1d: scattering coefficients");
        // boundary values (2 per step)
        std::vector<int> len(count);
        for (int i = 0; i < count; ++i) len[i] = 2;
        LSS_CUDA_TRY(d_len.alloc(count), "heat1d: set-up");
        LSS_CUDA_TRY(d_len.upload(len.data(), count), "heat1d: set-up");
        LSS_CUDA_TRY(d_off.upload(bnd_off.data(), count), "heat1d: set-up");
        LSS_CUDA_TRY(d_flat.alloc(std::max(1LL, bpos)), "heat1d: set-up");
        LSS_CUDA_TRY(d_flat.upload(bnd_flat.data(), bpos), "heat1d: set-up");
        k_h1_scatter_rows<T><<<std::min(grid_for(bpos, 256), 65535), 256>>>(d_groups.p, d_ig.p, d_il.p, d_off.p,
                                                                           d_len.p, count, d_flat.p, d_bnd.p, 0, bpos);
        LSS_CUDA_TRY(cudaGetLastError(), "heat1d: scattering boundary values");
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "heat1d: scattering boundary values");
        if (spos > 0) {
            // instances without a source own no rows: give them an offset past the end so
            // that the search never lands on them for a position they do not own
            std::vector<long long> so(count);
            std::vector<int> sidx;
            for (int i = 0; i < count; ++i)
                if (info[i].has_src) sidx.push_back(i);
            std::vector<long long> soff(sidx.size());
            std::vector<int> sig(sidx.size()), sil(sidx.size()), sn(sidx.size());
            for (size_t j = 0; j < sidx.size(); ++j) {
                soff[j] = src_off[sidx[j]];
                sig[j] = inst_group[sidx[j]];
                sil[j] = inst_lane[sidx[j]];
                sn[j] = info[sidx[j]].n;
            }
            const int sc = static_cast<int>(sidx.size());
            LSS_CUDA_TRY(d_off.upload(soff.data(), sc), "heat1d: set-up");
            LSS_CUDA_TRY(d_ig.upload(sig.data(), sc), "heat1d: set-up");
            LSS_CUDA_TRY(d_il.upload(sil.data(), sc), "heat1d: set-up");
            LSS_CUDA_TRY(d_len.upload(sn.data(), sc), "heat1d: set-up");
            LSS_CUDA_TRY(d_flat.alloc(spos), "heat1d: set-up");
            LSS_CUDA_TRY(d_flat.upload(src_flat.data(), spos), "heat1d: set-up");
            k_h1_scatter_rows<T><<<std::min(grid_for(spos, 256), 65535), 256>>>(
                d_groups.p, d_ig.p, d_il.p, d_off.p, d_len.p, sc, d_flat.p, d_src.p, 1, spos);
            LSS_CUDA_TRY(cudaGetLastError(), "heat1d: scattering source rows");
            LSS_CUDA_TRY(cudaDeviceSynchronize(), "heat1d: scattering source rows");
        }
    }
    if (arith == LSS_ADI_ARITH_FAST) {
        int dev = 0, sms = 0;
        LSS_CUDA_TRY(cudaGetDevice(&dev), "heat1d: device");
        LSS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "heat1d: SM count");
        std::vector<double> work(groups.size());
        for (size_t g = 0; g < groups.size(); ++g) work[g] = static_cast<double>(groups[g].n) * groups[g].steps;
        sched = schedule_groups(work, sms, h1_warps<T>());
        LSS_CUDA_TRY(d_wfirst.alloc(sched.first.size()), "heat1d: allocating the warp schedule");
        LSS_CUDA_TRY(d_wfirst.upload(sched.first.data(), sched.first.size()), "heat1d: uploading the warp schedule");
        LSS_CUDA_TRY(d_wgroup.alloc(sched.group.size()), "heat1d: allocating the warp schedule");
        LSS_CUDA_TRY(d_wgroup.upload(sched.group.data(), sched.group.size()), "heat1d: uploading the warp schedule");
        const h1params<T> p = params();
        k_h1_setup_fast<T><<<grid_for(static_cast<long long>(groups.size()) * LANES, 128), 128>>>(p);
        LSS_CUDA_TRY(cudaGetLastError(), "heat1d: launching the factorisation");
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "heat1d: factorisation");
    }
    return LSS_ADI_OK;
}

template <typename T> int batch_t<T>::run(cudaStream_t s)
{
    const h1params<T> p = params();
    const int blocks = grid_for(static_cast<long long>(groups.size()) * LANES, 128);
    const bool keep = d_all.p != nullptr, src = d_src.p != nullptr;
    if (arith == LSS_ADI_ARITH_FAST) {
        const int ctas = sched.ctas, th = h1_warps<T>() * LANES;
        if (keep && src) k_h1_fast<T, H1_PF, true, true><<<ctas, th, 0, s>>>(p);
        else if (keep) k_h1_fast<T, H1_PF, false, true><<<ctas, th, 0, s>>>(p);
        else if (src) k_h1_fast<T, H1_PF, true, false><<<ctas, th, 0, s>>>(p);
        else k_h1_fast<T, H1_PF, false, false><<<ctas, th, 0, s>>>(p);
    }
    else if (ds)
        k_h1_ref<T, true, 4><<<blocks, 128, 0, s>>>(p);
    else
        k_h1_ref<T, false, 4><<<blocks, 128, 0, s>>>(p);
    LSS_CUDA_TRY(cudaGetLastError(), "heat1d: launching the time loop");
    return LSS_ADI_OK;
}

// ---- Black-Scholes tables in the reference's arithmetic (host) ----------------------------
// grid_config_1d (discretization/lss_grid_config.hpp:21-52), grid_transform_config<One>
// (discretization/lss_grid_transform_config.hpp:32-87), heat_data_transform<One>
// (pde_solvers/transformation/lss_heat_data_transform.hpp:34-131), general_heat_equation_coefficients
// (implicit_coefficients/lss_1d_general_heat_equation_coefficients.hpp:34-64); user lambdas as in
// unit_tests/pde_solvers/one_dimensional/lss_black_scholes_equation_t.hpp:854-880 (double).
template <typename T> static void bs_tables(const lss_heat1d_bs &q, host_tables<T> &tb, inst_info &f)
{
    const int n = q.n, steps = q.nt - 1;
    const T one = T(1.0), two = T(2.0), half = T(0.5);
    const T step = one / static_cast<T>(static_cast<size_t>(n - 1));
    const T k = (static_cast<T>(q.maturity) - T(0.0)) / static_cast<T>(static_cast<size_t>(q.nt - 1));
    const T h = one / static_cast<T>(static_cast<size_t>(n - 1));
    const T lambda = k / (h * h), gamma = k / (two * h), delta = half * k;
    const T low = static_cast<T>(q.s_lo), high = static_cast<T>(q.s_hi), point = static_cast<T>(q.acc_point);
    T alpha = high - low;
    if (q.nonuniform) alpha = (point - low) / static_cast<T>(q.alpha_scale);
    const T c0 = std::asinh((high - point) / alpha), c1 = std::asinh((low - point) / alpha);
    const T cdiff = c0 - c1;
    auto arg = [&](T z) { return c0 * z + c1 * (one - z); };
    auto xval = [&](T z) { return point + alpha * std::sinh(arg(z)); };
    auto ader = [&](T z) { return alpha * cdiff * std::cosh(arg(z)); };
    auto bder = [&](T z) { return alpha * cdiff * cdiff * std::sinh(arg(z)); };
    const double sig = q.sigma, rate = q.rate, strike = q.strike, maturity = q.maturity, s_hi = q.s_hi;
    auto ua = [&](T x) -> T { return static_cast<T>(0.5 * sig * sig * x * x); };
    auto ub = [&](T x) -> T { return static_cast<T>(rate * x); };
    auto uc = [&](T x) -> T { (void)x; return static_cast<T>(-rate); };
    tb.coef.resize(3 * static_cast<size_t>(n));
    tb.init.resize(n);
    tb.x.resize(n);
    for (int i = 0; i < n; ++i) {
        const T zeta = step * static_cast<T>(static_cast<size_t>(i));
        const T x = xval(zeta);
        const T av = ader(zeta);
        const T ta = ua(x) / (ader(zeta) * ader(zeta));
        const T first = ub(x) / av;
        const T second = (ua(x) * bder(zeta)) / (av * av * av);
        const T tbv = first - second;
        const T tc = uc(x);
        tb.coef[i] = lambda * ta - gamma * tbv;
        tb.coef[n + i] = lambda * ta - delta * tc;
        tb.coef[2 * n + i] = lambda * ta + gamma * tbv;
        const T v = q.put ? static_cast<T>(strike - static_cast<double>(x)) : static_cast<T>(static_cast<double>(x) - strike);
        tb.init[i] = (T(0.0) < v) ? v : T(0.0);
        tb.x[i] = x;
    }
    // boundary values at the times of the backward loop: t = maturity - k, then -= k
    tb.bnd.resize(2 * static_cast<size_t>(steps));
    T time = static_cast<T>(q.maturity) - k;
    for (int s = 0; s < steps; ++s) {
        const double disc = strike * std::exp(-rate * (maturity - static_cast<double>(time)));
        tb.bnd[2 * s] = q.put ? static_cast<T>(disc) : T(0.0);
        tb.bnd[2 * s + 1] = q.put ? T(0.0) : static_cast<T>(s_hi - disc);
        time -= k;
    }
    f.n = n;
    f.nt = q.nt;
    f.lo_kind = f.hi_kind = LSS_HEAT1D_DIRICHLET;
    f.has_src = 0;
    f.forward = 0;
    f.theta_scheme = q.theta_scheme;
    f.t_lo = 0.0;
    f.t_hi = q.maturity;
    f.lo_lin = f.hi_lin = 0.0;
    // linear interpolation weight of eval_s
    int i0 = 0;
    while (i0 + 2 < n && static_cast<double>(tb.x[i0 + 1]) <= q.eval_s) ++i0;
    const double x0 = static_cast<double>(tb.x[i0]), x1 = static_cast<double>(tb.x[i0 + 1]);
    f.eval_i = i0;
    f.eval_w = x1 > x0 ? std::min(1.0, std::max(0.0, (q.eval_s - x0) / (x1 - x0))) : 0.0;
}

} // namespace heat1d
} // namespace lss_gb300

using namespace lss_gb300;
using namespace lss_gb300::heat1d;

struct lss_heat1d_batch {
    std::unique_ptr<batch_base> impl;
    cudaStream_t last = nullptr;
};

template <typename T> static batch_t<T> *as(lss_heat1d_batch *b) { return static_cast<batch_t<T> *>(b->impl.get()); }

static int valid_common(int count, int precision, int arith, int options, lss_heat1d_batch **b)
{
    if (!b) return set_error(LSS_ADI_EINVAL, "heat1d: batch pointer is NULL");
    *b = nullptr;
    if (count < 1) return set_error(LSS_ADI_EINVAL, "heat1d: count must be >= 1");
    if (precision != LSS_ADI_FP64 && precision != LSS_ADI_FP32) return set_error(LSS_ADI_EINVAL, "heat1d: precision");
    if (arith != LSS_ADI_ARITH_FAST && arith != LSS_ADI_ARITH_REFERENCE) return set_error(LSS_ADI_EINVAL, "heat1d: arith");
    if (options & ~(LSS_HEAT1D_OPT_ALL_STEPS | LSS_HEAT1D_OPT_DOUBLE_SWEEP))
        return set_error(LSS_ADI_EINVAL, "heat1d: unknown option bits");
    return LSS_ADI_OK;
}

template <typename T>
static int create_tab(const lss_heat1d_tables *ps, int count, int arith, int options, lss_heat1d_batch **b)
{
    std::vector<inst_info> info(count);
    std::vector<host_tables<T>> tabs(count);
    for (int i = 0; i < count; ++i) {
        const lss_heat1d_tables &q = ps[i];
        if (q.n < 4 || q.nt < 2) return set_error(LSS_ADI_EINVAL, "heat1d: n must be >= 4 and nt >= 2");
        if (!check_theta(q.theta_scheme))
            return set_error(LSS_ADI_EINVAL, "heat1d: the implicit 1-D kernel accepts Euler and Crank-Nicolson only");
        if (q.lo_kind < 0 || q.lo_kind > 2 || q.hi_kind < 0 || q.hi_kind > 2)
            return set_error(LSS_ADI_EINVAL, "heat1d: unknown boundary kind");
        if (!q.coef || !q.initial || !q.boundary) return set_error(LSS_ADI_EINVAL, "heat1d: table pointer is NULL");
        if (!(q.t_hi > q.t_lo)) return set_error(LSS_ADI_EINVAL, "heat1d: t_hi must exceed t_lo");
        const int n = q.n, steps = q.nt - 1;
        const T *coef = static_cast<const T *>(q.coef), *init = static_cast<const T *>(q.initial);
        const T *bnd = static_cast<const T *>(q.boundary);
        host_tables<T> &tb = tabs[i];
        tb.coef.assign(coef, coef + 3 * static_cast<size_t>(n));
        tb.init.assign(init, init + n);
        tb.bnd.resize(2 * static_cast<size_t>(steps));
        for (int s = 0; s < steps; ++s) {
            if (bnd[4 * s + 1] != bnd[1] || bnd[4 * s + 3] != bnd[3])
                return set_error(LSS_ADI_EUNSUPPORTED, "heat1d: Robin linear values must not change in time");
            tb.bnd[2 * s] = bnd[4 * s];
            tb.bnd[2 * s + 1] = bnd[4 * s + 2];
        }
        if (q.source) {
            const T *src = static_cast<const T *>(q.source);
            tb.src.assign(src, src + static_cast<size_t>(q.nt) * n);
        }
        inst_info &f = info[i];
        f.n = n;
        f.nt = q.nt;
        f.lo_kind = q.lo_kind;
        f.hi_kind = q.hi_kind;
        f.has_src = q.source ? 1 : 0;
        f.forward = q.forward ? 1 : 0;
        f.theta_scheme = q.theta_scheme;
        f.t_lo = q.t_lo;
        f.t_hi = q.t_hi;
        f.lo_lin = q.lo_kind == LSS_HEAT1D_ROBIN ? static_cast<double>(bnd[1]) : 0.0;
        f.hi_lin = q.hi_kind == LSS_HEAT1D_ROBIN ? static_cast<double>(bnd[3]) : 0.0;
        f.eval_i = n / 2; // value = the solution's middle point (n >= 4: n/2 + 1 < n)
        f.eval_w = 0.0;
    }
    auto bt = std::make_unique<batch_t<T>>();
    bt->precision = std::is_same<T, double>::value ? LSS_ADI_FP64 : LSS_ADI_FP32;
    bt->arith = arith;
    bt->options = options;
    bt->ds = (options & LSS_HEAT1D_OPT_DOUBLE_SWEEP) != 0;
    int rc = bt->build(std::move(info), tabs);
    if (rc != LSS_ADI_OK) return rc;
    auto *h = new (std::nothrow) lss_heat1d_batch;
    if (!h) return set_error(LSS_ADI_ENOMEM, "heat1d: host allocation");
    h->impl = std::move(bt);
    *b = h;
    return LSS_ADI_OK;
}

template <typename T>
static int create_bs(const lss_heat1d_bs *ps, int count, int arith, int options, lss_heat1d_batch **b)
{
    for (int i = 0; i < count; ++i) {
        const lss_heat1d_bs &q = ps[i];
        if (q.n < 4 || q.nt < 2) return set_error(LSS_ADI_EINVAL, "heat1d: n must be >= 4 and nt >= 2");
        if (!check_theta(q.theta_scheme))
            return set_error(LSS_ADI_EINVAL, "heat1d: the implicit 1-D kernel accepts Euler and Crank-Nicolson only");
        if (!(q.s_hi > q.s_lo) || !(q.maturity > 0.0) || !(q.sigma > 0.0))
            return set_error(LSS_ADI_EINVAL, "heat1d: invalid Black-Scholes problem (ranges, maturity, sigma)");
        if (q.nonuniform && !(q.alpha_scale > 0.0)) return set_error(LSS_ADI_EINVAL, "heat1d: alpha_scale must be > 0");
    }
    std::vector<inst_info> info(count);
    std::vector<host_tables<T>> tabs(count);
    const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    const int nthr = static_cast<int>(std::min<long long>(hw, count));
    std::vector<std::thread> pool;
    for (int w = 0; w < nthr; ++w)
        pool.emplace_back([&, w]() {
            for (int i = w; i < count; i += nthr) bs_tables<T>(ps[i], tabs[i], info[i]);
        });
    for (auto &t : pool) t.join();
    auto bt = std::make_unique<batch_t<T>>();
    bt->precision = std::is_same<T, double>::value ? LSS_ADI_FP64 : LSS_ADI_FP32;
    bt->arith = arith;
    bt->options = options;
    bt->ds = (options & LSS_HEAT1D_OPT_DOUBLE_SWEEP) != 0;
    int rc = bt->build(std::move(info), tabs);
    if (rc != LSS_ADI_OK) return rc;
    auto *h = new (std::nothrow) lss_heat1d_batch;
    if (!h) return set_error(LSS_ADI_ENOMEM, "heat1d: host allocation");
    h->impl = std::move(bt);
    *b = h;
    return LSS_ADI_OK;
}

template <typename T> static int run_host_t(lss_heat1d_batch *b, const void *initials, double *values, int *status,
                                            cudaStream_t s)
{
    batch_t<T> *bt = as<T>(b);
    if (initials)
        LSS_CUDA_TRY(cudaMemcpyAsync(bt->d_init.p, initials, bt->total_init * sizeof(T), cudaMemcpyHostToDevice, s),
                     "heat1d: uploading initial conditions");
    int rc = bt->run(s);
    if (rc) return rc;
    if (values)
        LSS_CUDA_TRY(cudaMemcpyAsync(values, bt->d_values.p, bt->count * sizeof(double), cudaMemcpyDeviceToHost, s),
                     "heat1d: downloading values");
    if (status)
        LSS_CUDA_TRY(cudaMemcpyAsync(status, bt->d_status.p, bt->count * sizeof(int), cudaMemcpyDeviceToHost, s),
                     "heat1d: downloading status");
    LSS_CUDA_TRY(cudaStreamSynchronize(s), "heat1d: end-to-end step");
    return LSS_ADI_OK;
}

template <typename T> static int solution_t(lss_heat1d_batch *b, int index, void *out)
{
    batch_t<T> *bt = as<T>(b);
    const int gi = bt->inst_group[index], lane = bt->inst_lane[index];
    const h1group &G = bt->groups[gi];
    const inst_info &f = bt->info[index];
    const bool all = (bt->options & LSS_HEAT1D_OPT_ALL_STEPS) != 0;
    const long long rows = all ? f.nt : 1;
    const long long src_off = all ? G.all : G.pt + static_cast<long long>(S_U) * G.n * LANES;
    const T *src = all ? bt->d_all.p : bt->d_pt.p;
    // strided copy: element t of row r at src_off + (r*n + t)*32 + lane
    LSS_CUDA_TRY(cudaMemcpy2D(out, sizeof(T), src + src_off + lane, LANES * sizeof(T), sizeof(T), rows * f.n,
                              cudaMemcpyDeviceToHost),
                 "heat1d: downloading a solution");
    return LSS_ADI_OK;
}

extern "C" {

int lss_heat1d_batch_create(const lss_heat1d_tables *problems, int count, int precision, int arith, int options,
                            lss_heat1d_batch **b)
{
    clear_error();
    int rc = valid_common(count, precision, arith, options, b);
    if (rc) return rc;
    if (!problems) return set_error(LSS_ADI_EINVAL, "heat1d: problems is NULL");
    try {
        return precision == LSS_ADI_FP64 ? create_tab<double>(problems, count, arith, options, b)
                                         : create_tab<float>(problems, count, arith, options, b);
    } catch (const std::bad_alloc &) {
        return set_error(LSS_ADI_ENOMEM, "heat1d: host allocation failed");
    }
}

int lss_heat1d_batch_create_bs(const lss_heat1d_bs *problems, int count, int precision, int arith, int options,
                               lss_heat1d_batch **b)
{
    clear_error();
    int rc = valid_common(count, precision, arith, options, b);
    if (rc) return rc;
    if (!problems) return set_error(LSS_ADI_EINVAL, "heat1d: problems is NULL");
    try {
        return precision == LSS_ADI_FP64 ? create_bs<double>(problems, count, arith, options, b)
                                         : create_bs<float>(problems, count, arith, options, b);
    } catch (const std::bad_alloc &) {
        return set_error(LSS_ADI_ENOMEM, "heat1d: host allocation failed");
    }
}

int lss_heat1d_batch_run(lss_heat1d_batch *b, void *stream)
{
    if (!b) return set_error(LSS_ADI_EINVAL, "heat1d: batch is NULL");
    clear_error();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    b->last = s;
    return b->impl->precision == LSS_ADI_FP64 ? as<double>(b)->run(s) : as<float>(b)->run(s);
}

int lss_heat1d_batch_run_host(lss_heat1d_batch *b, const void *initials, double *values, int *status, void *stream)
{
    if (!b) return set_error(LSS_ADI_EINVAL, "heat1d: batch is NULL");
    clear_error();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    b->last = s;
    return b->impl->precision == LSS_ADI_FP64 ? run_host_t<double>(b, initials, values, status, s)
                                              : run_host_t<float>(b, initials, values, status, s);
}

int lss_heat1d_batch_results(lss_heat1d_batch *b, double *values, int *status)
{
    if (!b) return set_error(LSS_ADI_EINVAL, "heat1d: batch is NULL");
    clear_error();
    LSS_CUDA_TRY(cudaStreamSynchronize(b->last), "heat1d: waiting for the run");
    const int count = b->impl->count;
    if (b->impl->precision == LSS_ADI_FP64) {
        auto *bt = as<double>(b);
        if (values) LSS_CUDA_TRY(cudaMemcpy(values, bt->d_values.p, count * sizeof(double), cudaMemcpyDeviceToHost), "heat1d: values");
        if (status) LSS_CUDA_TRY(cudaMemcpy(status, bt->d_status.p, count * sizeof(int), cudaMemcpyDeviceToHost), "heat1d: status");
    } else {
        auto *bt = as<float>(b);
        if (values) LSS_CUDA_TRY(cudaMemcpy(values, bt->d_values.p, count * sizeof(double), cudaMemcpyDeviceToHost), "heat1d: values");
        if (status) LSS_CUDA_TRY(cudaMemcpy(status, bt->d_status.p, count * sizeof(int), cudaMemcpyDeviceToHost), "heat1d: status");
    }
    return LSS_ADI_OK;
}

int lss_heat1d_batch_solution(lss_heat1d_batch *b, int index, void *out)
{
    if (!b || !out) return set_error(LSS_ADI_EINVAL, "heat1d: NULL argument");
    if (index < 0 || index >= b->impl->count) return set_error(LSS_ADI_EINVAL, "heat1d: index out of range");
    clear_error();
    LSS_CUDA_TRY(cudaStreamSynchronize(b->last), "heat1d: waiting for the run");
    return b->impl->precision == LSS_ADI_FP64 ? solution_t<double>(b, index, out) : solution_t<float>(b, index, out);
}

int lss_heat1d_batch_grid(const lss_heat1d_batch *b, int index, void *x)
{
    if (!b || !x) return set_error(LSS_ADI_EINVAL, "heat1d: NULL argument");
    if (index < 0 || index >= b->impl->count) return set_error(LSS_ADI_EINVAL, "heat1d: index out of range");
    if (b->impl->precision == LSS_ADI_FP64) {
        auto *bt = static_cast<const batch_t<double> *>(b->impl.get());
        if (bt->grids.size() != static_cast<size_t>(bt->count)) return set_error(LSS_ADI_EINVAL, "heat1d: not a Black-Scholes batch");
        std::copy(bt->grids[index].begin(), bt->grids[index].end(), static_cast<double *>(x));
    } else {
        auto *bt = static_cast<const batch_t<float> *>(b->impl.get());
        if (bt->grids.size() != static_cast<size_t>(bt->count)) return set_error(LSS_ADI_EINVAL, "heat1d: not a Black-Scholes batch");
        std::copy(bt->grids[index].begin(), bt->grids[index].end(), static_cast<float *>(x));
    }
    return LSS_ADI_OK;
}

int lss_heat1d_batch_launch_count(const lss_heat1d_batch *b) { return b ? 1 : 0; }

double lss_heat1d_batch_point_steps(const lss_heat1d_batch *b) { return b ? b->impl->point_steps : 0.0; }

void lss_heat1d_batch_destroy(lss_heat1d_batch *b) { delete b; }

} // extern "C"
