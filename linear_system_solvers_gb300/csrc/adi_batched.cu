// adi_batched.cu -- many uneven ADI instances advanced by one persistent kernel.
//
// Each CTA is cut into warp groups of 1-4 warps; a group pulls an instance index from its
// class's device counter (instances sorted longest first), runs that instance's whole time
// loop with the group's own barrier between the sweeps, then pulls the next one.  The
// time-invariant line systems of every instance are
// factorised once on the device (k_setup_s_lines / k_setup_v_lines): the time loop only
// does the pre-scaled right-hand side, one FMA of forward recurrence and one of back
// substitution per point, because GB300's FP64 pipe (~1.25 TFLOP/s measured) and not HBM
// is the binding resource.  Same time-step structure as the reference
// (implicit_heston_time_loop::run, lss_2d_general_heston_equation_implicit_kernel.hpp:150-207).
#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "adi_batched.hpp"

namespace lss_gb300 {

// slots of the S-direction tables ([t][j] layout, n = nx*ny per slot)
enum {
    SL_LA = 0, SL_G, SL_WG, SL_WW, SL_WS, SL_WC, SL_WN, SL_WE,
    SL_S2SC, SL_S2SE, SL_S2IB, SL_S2MZ, SL_X1, SL_X2, SL_X3, SL_X4, SL_X5, SL_IB, SL_COUNT
};
// slots of the v-direction tables ([t][i] layout: i fastest)
enum { VL_LA = 0, VL_G, VL_VC, VL_VN, VL_IB, VL_COUNT };
// per-instance 1-D arrays along S (nx each).  Adjoint only, coefficient derivatives split into
// S and v factors: X_HX = S/A (dd^/dr), X_HC = S-factor of c^ (Heston S/A, SABR F^beta/A),
// X_HA = F^(2 beta)/A^2 and X_HDD = F^(2 beta) A''/A^3 (SABR D(t) terms of a^ and d^)
enum { XB_M = 0, XB_C, XB_P, XB_2, XB_1, X_VHI, X_CHV, X_HX, X_HC, X_HA, X_HDD, X_COUNT };
// per-instance 1-D arrays along v (ny each).  Adjoint only: Y_HY = v-factor of c^ (Heston v/B,
// SABR v^2/B), Y_BS = db^/dsigma, Y_EK = de^/dkappa, Y_ET = de^/dtheta, Y_ES = de^/dsigma,
// Y_HV2 = v^2/2 (SABR D(t) terms)
enum { Y_SLO = 0, Y_B2C, Y_CHS, Y_HY, Y_BS, Y_EK, Y_ET, Y_ES, Y_HV2, Y_COUNT };

struct bdesc {
    int nx, ny, steps, scheme;
    long long o2;  // offset of the instance in the nx*ny arenas
    int ox, oy;    // offsets in the nx- and ny-sized arenas
    double bnc;    // constant of the Neumann-corner boundary row
    int i0, j0;    // bilinear cell of (eval_s, eval_v)
    double w00, w10, w01, w11;
    int ck;        // checkpoint interval of the adjoint (steps)
    int pad_;
    // scalars of the parameter derivatives: delta, k/2, ni, beta~, sigma, rho, theta, zeta, gamma, k
    double a_delta, a_halfk, a_ni, a_betat, a_sigma, a_rho, a_theta, a_zeta, a_gamma, a_k;
    // SABR (r = 0): dD^p/dr = -p tau with tau = T - t = a_tau0 + a_dtau * step; alpha~, 1 - beta
    int model, pad2_;
    double a_alphat, a_omb, a_tau0, a_dtau;
};

// Instances are split into classes by the number of warps that work on one of them (1..4 for
// the persistent kernels: about one thread per S line).  Class c's instances are
// order[cls_start[c] .. cls_start[c] + cls_count[c]), longest first, pulled through counter[c].
constexpr int MAX_GROUP_WARPS = 4;

// Most chunks per line of the partitioned line solves of one large instance (wide path): a CTA
// holds L lines x P chunks (L * P <= 1024 threads) and composes the chunks' carries through two
// shared arrays of 1024 values, indexed [chunk][line] (carry2d).
constexpr int MAX_CHUNKS = 128;
template <typename T> struct carry2d {
    T *p;
    int L; // lines per CTA (blockDim.x)
    __device__ __forceinline__ T *operator[](int c) const { return p + c * L; }
};

template <typename T> struct bparams {
    const bdesc *desc;
    const int *order;
    int count;
    int *counter;                     // one work counter per class (index 1..4)
    int cls_start[MAX_GROUP_WARPS + 1], cls_count[MAX_GROUP_WARPS + 1];
    long long cls_need[MAX_GROUP_WARPS + 1]; // largest adjoint workspace (doubles) of a class's instances
    const int *layout;                // per CTA: sizes of its warp groups, one hex digit each, lowest first
    T *U, *V, *Y1, *Y2, *Y3;          // state arenas (sum nx*ny each)
    T *B0;                            // nx arena: the explicit v = v_lo boundary column of a step
    const T *S[SL_COUNT];             // S-direction tables
    const T *Vt[VL_COUNT];            // v-direction tables
    const T *X[X_COUNT];              // nx arenas
    const T *Yv[Y_COUNT];             // ny arenas
    const int *imap, *jmap;           // nx / ny arenas
    double *values;                   // count
    int *status;                      // count
    int *final_in_v;                  // count: 1 if the final surface is in V
    // forward + adjoint (mode 1, FP64 only)
    double *grads;                    // 5 * count: d value / d(kappa, theta, sigma, rho, r)
    double *ws;                       // adjoint workspace: a slice of ws_per_warp doubles per warp
    long long ws_per_warp;            // a group of w warps owns w consecutive slices
    const T *payoff;                  // sum nx*ny initial conditions
};

// The warps of one CTA that work on one instance together, synchronised by their own named
// barrier (a one-warp group by __syncwarp), so that the groups of a CTA run independently.
struct grp {
    int t;      // thread index in the group
    int n;      // threads in the group (a multiple of 32)
    int gi;     // group index in the CTA (barrier 1 + gi)
    int warp0;  // first warp of the group in the CTA
    __device__ __forceinline__ void sync() const
    {
        // constant barrier ids: a run-time id makes the compiler reserve all 16 of the CTA's
        // named barriers, which would cap the CTAs per SM at 4
        if (n == 32) {
            __syncwarp();
        } else {
            switch (gi) {
            case 0: __barrier_sync_count(1, n); break;
            case 1: __barrier_sync_count(2, n); break;
            case 2: __barrier_sync_count(3, n); break;
            default: __barrier_sync_count(4, n); break;
            }
        }
    }
};

// This thread's group from the CTA's layout word (group sizes in warps, one hex digit each).
__device__ __forceinline__ grp make_grp(int layout)
{
    const int w = threadIdx.x >> 5;
    int first = 0, gi = 0, size = layout & 15;
    while (size > 0 && w >= first + size) {
        first += size;
        layout >>= 4;
        size = layout & 15;
        ++gi;
    }
    grp g;
    g.gi = gi;
    g.warp0 = first;
    g.n = 32 * (size > 0 ? size : 1);
    g.t = threadIdx.x - 32 * first;
    return g;
}

// Next instance for a group whose home class is `cls` (updated in place as classes run dry):
// its own class first, then the classes of fewer warps per instance; with max_need >= 0 only
// classes whose instances' workspace fits max_need doubles.  Called by the group's thread 0.
template <typename T>
__device__ __forceinline__ int next_instance(const bparams<T> &p, int &cls, long long max_need)
{
    while (cls >= 1) {
        if (p.cls_count[cls] > 0 && (max_need < 0 || p.cls_need[cls] <= max_need)) {
            const int q = atomicAdd(p.counter + cls, 1);
            if (q < p.cls_count[cls]) return p.order[p.cls_start[cls] + q];
        }
        --cls;
    }
    return -1;
}

// ------------------------------------------------------------------------------------------
// set-up: factorise the S-lines and v-lines of every instance once (double arithmetic)
// ------------------------------------------------------------------------------------------
struct setup_params {
    const bdesc *desc;
    const long long *line_start; // prefix of line counts per instance
    int count;
    long long total_lines;
    const double *base;          // 7 * sum(n): M, P, Z, Mt, Pt, W, C (each arena sum(n))
    long long total_n;
    const double *scal;          // per instance: theta, zeta, gamma
};

// The 18 S-line slots of one point from its coefficients, 1/beta and gamma (double arithmetic).
template <typename T>
__device__ __forceinline__ void s_line_slots(T *s, long long slot_stride, int scheme, double th, double ze, double gm,
                                             double M, double P, double Z, double Mt, double Pt, double W, double C,
                                             double ib, double gam)
{
    const double a = -th * M, c = -th * P;
    s[SL_LA * slot_stride] = static_cast<T>(a * ib);
    s[SL_G * slot_stride] = static_cast<T>(gam);
    s[SL_WG * slot_stride] = static_cast<T>(gm * C * ib);
    s[SL_WW * slot_stride] = static_cast<T>((1.0 - th) * M * ib);
    s[SL_WS * slot_stride] = static_cast<T>(Mt * ib);
    s[SL_WC * slot_stride] = static_cast<T>((1.0 - W - (1.0 - th) * Z) * ib);
    s[SL_WN * slot_stride] = static_cast<T>(Pt * ib);
    s[SL_WE * slot_stride] = static_cast<T>((1.0 - th) * P * ib);
    const double sc = th * Z * ib, se = c * ib;
    if (scheme == LSS_ADI_HUNDSDORFER_VERWER) {
        // fused HV stage: rhs4 + rhs_intermed_3 expressed in Delta = Y2 - U and Y1
        s[SL_S2SC * slot_stride] = static_cast<T>(sc + ib);
        s[SL_S2SE * slot_stride] = static_cast<T>(se);
        s[SL_S2IB * slot_stride] = static_cast<T>(0.0);
        s[SL_S2MZ * slot_stride] = static_cast<T>(ze * gm * C * ib);
        s[SL_X1 * slot_stride] = static_cast<T>(a * ib + ze * M * ib);
        s[SL_X2 * slot_stride] = static_cast<T>(sc - ze * (W + Z) * ib);
        s[SL_X3 * slot_stride] = static_cast<T>(se + ze * P * ib);
        s[SL_X4 * slot_stride] = static_cast<T>(ze * Mt * ib);
        s[SL_X5 * slot_stride] = static_cast<T>(ze * Pt * ib);
    } else {
        const double zt = (scheme == LSS_ADI_MODIFIED_CRAIG_SNEYD) ? (ze - th) : 0.0;
        s[SL_S2SC * slot_stride] = static_cast<T>(sc);
        s[SL_S2SE * slot_stride] = static_cast<T>(se);
        s[SL_S2IB * slot_stride] = static_cast<T>(ib);
        s[SL_S2MZ * slot_stride] = static_cast<T>(ze * gm * C * ib);
        s[SL_X1 * slot_stride] = static_cast<T>(zt * M * ib);
        s[SL_X2 * slot_stride] = static_cast<T>(-zt * (Z + W) * ib);
        s[SL_X3 * slot_stride] = static_cast<T>(-zt * P * ib);
        s[SL_X4 * slot_stride] = static_cast<T>(zt * Mt * ib);
        s[SL_X5 * slot_stride] = static_cast<T>(zt * Pt * ib);
    }
    s[SL_IB * slot_stride] = static_cast<T>(ib);
}

template <typename T>
__global__ void k_setup_s_lines(setup_params sp, T *S0, long long slot_stride, T *chS_arena)
{
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= sp.total_lines) return;
    int inst = 0;
    { // binary search the instance owning global line g
        int lo = 0, hi = sp.count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sp.line_start[mid] <= g) lo = mid; else hi = mid - 1;
        }
        inst = lo;
    }
    const bdesc d = sp.desc[inst];
    const int j = 1 + static_cast<int>(g - sp.line_start[inst]);
    const int nx = d.nx, ny = d.ny, e = nx - 2;
    const double th = sp.scal[3 * inst], ze = sp.scal[3 * inst + 1], gm = sp.scal[3 * inst + 2];
    const long long N = sp.total_n;
    const double *__restrict__ bM = sp.base, *__restrict__ bP = sp.base + N, *__restrict__ bZ = sp.base + 2 * N,
                 *__restrict__ bMt = sp.base + 3 * N, *__restrict__ bPt = sp.base + 4 * N,
                 *__restrict__ bW = sp.base + 5 * N, *__restrict__ bC = sp.base + 6 * N;
    // the next point's coefficients are loaded before this point's eighteen stores, so that one
    // DRAM latency per point overlaps the work of the point before (the loop is serial along the
    // line: the set-up of one instance's lines runs on few threads before every step of a
    // time-dependent instance)
    long long o1 = d.o2 + ny + j;
    double nM = bM[o1], nP = bP[o1], nZ = bZ[o1], nMt = bMt[o1], nPt = bPt[o1], nW = bW[o1], nC = bC[o1];
    double gam = 0.0;
    for (int t = 1; t <= e; ++t) {
        const long long o = d.o2 + (long long)t * ny + j;
        const double M = nM, P = nP, Z = nZ, Mt = nMt, Pt = nPt, W = nW, C = nC;
        if (t < e) {
            o1 = o + ny;
            nM = bM[o1]; nP = bP[o1]; nZ = bZ[o1]; nMt = bMt[o1]; nPt = bPt[o1]; nW = bW[o1]; nC = bC[o1];
        }
        const double a = -th * M, b = 1.0 + th * Z, c = -th * P;
        const double beta = (t == 1) ? b : b - a * gam;
        const double ib = 1.0 / beta;
        if (t < e) gam = c / beta;
        s_line_slots<T>(S0 + o, slot_stride, d.scheme, th, ze, gm, M, P, Z, Mt, Pt, W, C, ib, t < e ? gam : 0.0);
        if (t == e) chS_arena[d.oy + j] = static_cast<T>(c * ib);
    }
}

template <typename T>
__global__ void k_setup_v_lines(setup_params sp, T *V0, long long slot_stride, T *chV_arena)
{
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= sp.total_lines) return;
    int lo = 0, hi = sp.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sp.line_start[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const int inst = lo;
    const bdesc d = sp.desc[inst];
    const int i = 1 + static_cast<int>(g - sp.line_start[inst]);
    const int nx = d.nx, ny = d.ny, e = ny - 2;
    const double th = sp.scal[3 * inst];
    const long long N = sp.total_n;
    const double *bMt = sp.base + 3 * N, *bPt = sp.base + 4 * N, *bW = sp.base + 5 * N;
    double gam = 0.0;
    for (int t = 1; t <= e; ++t) {
        const long long ob = d.o2 + (long long)i * ny + t;  // base tables are [i][j]
        const long long o = d.o2 + (long long)t * nx + i;   // v tables are [t][i]
        const double a = -th * bMt[ob], b = 1.0 + th * bW[ob], c = -th * bPt[ob];
        const double beta = (t == 1) ? b : b - a * gam;
        const double ib = 1.0 / beta;
        if (t < e) gam = c / beta;
        T *s = V0 + o;
        s[VL_LA * slot_stride] = static_cast<T>(a * ib);
        s[VL_G * slot_stride] = static_cast<T>(t < e ? gam : 0.0);
        s[VL_VC * slot_stride] = static_cast<T>(th * bW[ob] * ib);
        s[VL_VN * slot_stride] = static_cast<T>(c * ib);
        s[VL_IB * slot_stride] = static_cast<T>(ib);
        if (t == e) chV_arena[d.ox + i] = static_cast<T>(c * ib);
    }
}

// ------------------------------------------------------------------------------------------
// time-dependent coefficients of one instance (SABR with r != 0 on the wide kernels)
// ------------------------------------------------------------------------------------------
// a and c carry D(t)^(2(1-beta)) and D(t)^(1-beta), D(t) = exp(-r (T - t)); b, d, e, f do not.
// Before each step the S-direction base tables M, P, Z, C are re-evaluated at the step's powers
// da, dc (general_heston_equation_coefficients, coefficients.hpp:89-98, on the transformed data
// of lss_heat_data_transform.hpp:174-214) and the S lines re-factorised (k_tdep_s_factor,
// k_tdep_s_slots); the v-direction tables do not change.  The same kernel scales the S-factors of the adjoint's
// D(t) terms (X_HA, X_HDD by da, X_HC by dc) and the boundary-column weights that carry d^ on
// the v = v_lo line (XB_M, XB_P), so that the adjoint steps see this step's a^ and c^.
struct tdep_params {
    const double *a_static, *c_static, *ab; // n each: ((0.5 v) v) S^(2 beta), ((rho nu) v) v S^beta, A B
    const double *per_i;                    // 5 nx: A, A^2, A^3, A'', user d
    const double *xs;                       // 3 nx: X_HA, X_HDD, X_HC at D = 1
    double *base;                           // 7 n: M, P, Z, Mt, Pt, W, C
    long long n;
    int nx, ny;
    double alpha, delta, two_alpha, half_rho_f;
};

// The S-line factorisation of the time-dependent instance in two kernels: the recurrence
// beta_t = b_t - a_t gamma_{t-1} for 1/beta and gamma (k_tdep_s_factor, partitioned along the
// lines), then every slot of every point in parallel (s_line_slots, the same formulas as
// k_setup_s_lines).
template <typename T>
__global__ void k_tdep_s_slots(const double *__restrict__ base, long long n, int nx, int ny, int scheme, double th,
                               double ze, double gm, T *S0, T *chS)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int e = nx - 2;
    if (q >= (long long)e * (ny - 2)) return;
    const int t = 1 + static_cast<int>(q / (ny - 2)), j = 1 + static_cast<int>(q % (ny - 2));
    const long long o = (long long)t * ny + j;
    const double M = base[o], P = base[n + o], Z = base[2 * n + o], Mt = base[3 * n + o], Pt = base[4 * n + o],
                 W = base[5 * n + o], C = base[6 * n + o];
    const double ib = static_cast<double>(S0[SL_IB * n + o]), gam = static_cast<double>(S0[SL_G * n + o]);
    s_line_slots<T>(S0 + o, n, scheme, th, ze, gm, M, P, Z, Mt, Pt, W, C, ib, gam);
    if (t == e) chS[j] = static_cast<T>(-th * P * ib);
}

template <typename T>
__global__ void k_tdep_refresh(tdep_params tp, double da, double dc, T *xarena, long long total_x)
{
    const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= tp.n) return;
    const int nx = tp.nx, ny = tp.ny;
    const int i = static_cast<int>(o / ny), j = static_cast<int>(o % ny);
    const double aval = tp.per_i[i], aa = tp.per_i[nx + i], aaa = tp.per_i[2 * nx + i];
    const double gc = tp.per_i[3 * nx + i], ud = tp.per_i[4 * nx + i];
    const double A = tp.a_static[o] * da;
    const double ah = A / aa;
    const double dh = ud / aval - (A * gc) / aaa;
    tp.base[o] = tp.alpha * ah - tp.delta * dh;
    tp.base[tp.n + o] = tp.alpha * ah + tp.delta * dh;
    tp.base[2 * tp.n + o] = tp.two_alpha * ah - tp.half_rho_f;
    tp.base[6 * tp.n + o] = (tp.c_static[o] * dc) / tp.ab[o];
    if (j == 0) {
        xarena[XB_M * total_x + i] = static_cast<T>(-tp.delta * dh);
        xarena[XB_P * total_x + i] = static_cast<T>(tp.delta * dh);
        xarena[X_HA * total_x + i] = static_cast<T>(tp.xs[i] * da);
        xarena[X_HDD * total_x + i] = static_cast<T>(tp.xs[nx + i] * da);
        xarena[X_HC * total_x + i] = static_cast<T>(tp.xs[2 * nx + i] * dc);
    }
}

// ------------------------------------------------------------------------------------------
// the persistent time-loop kernel
// ------------------------------------------------------------------------------------------
// One instance's view of the arenas.  The arena base pointers stay in the kernel's parameter
// space (__grid_constant__), so they cost no registers; only the offsets are carried.
template <typename T> struct inst_view {
    const bparams<T> *p;
    int nx, ny, e_s, e_v;
    long long o2;
    int ox, oy;
    __device__ __forceinline__ const T *S(int k) const { return p->S[k] + o2; }
    __device__ __forceinline__ const T *Vt(int k) const { return p->Vt[k] + o2; }
    __device__ __forceinline__ const T *X(int k) const { return p->X[k] + ox; }
    __device__ __forceinline__ const T *Yv(int k) const { return p->Yv[k] + oy; }
    __device__ __forceinline__ const int *imap() const { return p->imap + ox; }
    __device__ __forceinline__ const int *jmap() const { return p->jmap + oy; }
};

template <typename T> __device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

// Explicitly rounded products and fused multiply-adds.  The v-line recurrences run in several
// kernels (rows read in place, rows through shared-memory tiles, partitioned lines), and the
// autotuner may pick a different variant per instance; written with these, every variant rounds
// the same way whatever the compiler would contract, so they agree bit for bit.
__device__ __forceinline__ double mul_x(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_x(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double fma_x(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_x(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// One point of the v-line forward recurrence: y_t = la a0 + vc a1 + vn a2 + ib h - la y_{t-1}
// (a0, a1, a2: `in` at t-1, t, t+1; h: `inh` at t).
template <typename T> __device__ __forceinline__ T v_point(T la, T vc, T vn, T ib, T a0, T a1, T a2, T h, T y)
{
    T f = mul_x(la, a0);
    f = fma_x(vc, a1, f);
    f = fma_x(vn, a2, f);
    f = fma_x(ib, h, f);
    return fma_x(-la, y, f);
}

// boundary#1: the v = v_lo column, explicit (explicit_boundary.hpp:39-84); result in smem
// Work distribution of every stage: items l0, l0 + ls, ... (threads of one CTA in the
// batched kernel; all threads of a grid in the per-stage kernels of the wide path).
template <typename T>
__device__ __forceinline__ void b1_stage(const inst_view<T> &v, const T *__restrict__ U, T *__restrict__ sb0, double bnc,
                                         int l0, int ls)
{
    const int nx = v.nx, ny = v.ny, N = nx - 1;
    for (int i = l0; i < nx; i += ls) {
        T r;
        if (i == 0) {
            r = ldg(v.Yv(Y_SLO));
        } else if (i == N) {
            r = ldg(v.X(XB_C) + i) * U[(long long)N * ny] + ldg(v.X(XB_1) + i) * U[(long long)N * ny + 1] +
                ldg(v.X(XB_2) + i) * U[(long long)N * ny + 2] + static_cast<T>(bnc);
        } else {
            const long long o = (long long)i * ny;
            r = ldg(v.X(XB_M) + i) * U[o - ny] + ldg(v.X(XB_C) + i) * U[o] + ldg(v.X(XB_P) + i) * U[o + ny] +
                ldg(v.X(XB_2) + i) * U[o + 2] + ldg(v.X(XB_1) + i) * U[o + 1];
        }
        sb0[i] = r;
    }
}

// boundary#2: row S_lo and the S_max extrapolation row (explicit_boundary.hpp:202-238)
template <typename T> __device__ __forceinline__ void b2_stage(const inst_view<T> &v, T *Vn, int l0, int ls)
{
    const int nx = v.nx, ny = v.ny, lri = nx - 1;
    const T four3 = T(4.0 / 3.0), third = T(1.0 / 3.0);
    for (int j = l0; j < ny; j += ls) {
        Vn[j] = ldg(v.Yv(Y_SLO) + j);
        const int jj = ldg(v.jmap() + j);
        Vn[(long long)lri * ny + j] =
            four3 * Vn[(long long)(lri - 1) * ny + jj] - third * Vn[(long long)(lri - 2) * ny + jj] - ldg(v.Yv(Y_B2C) + j);
    }
}

// S-line sweeps.  KIND 1: explicit operator on U (Y1).  KIND 2: second S stage of CS/MCS/HV
// (scheme SCH) on U, Y1, Y2.  Thread per line j; every access of a warp is one coalesced row
// segment.  The mixed difference (x(t-1,j-1) - x(t-1,j+1)) - (x(t+1,j-1) - x(t+1,j+1)) is formed
// from a rolling window of the per-row differences x(r,j-1) - x(r,j+1): one subtraction per row.
//
// s_line_fwd: right-hand side and forward recurrence y_t = f_t - la_t y_{t-1} of line j over
// rows t0..t1, starting from y = y_{t0-1}; writes y_t into Y and returns y_{t1}.
template <typename T, int KIND, int SCH>
__device__ __forceinline__ T s_line_fwd(const inst_view<T> &v, const T *__restrict__ U, const T *__restrict__ Y1,
                                        const T *__restrict__ Y2, T *__restrict__ Y, int j, int t0, int t1, T y, T hi)
{
    const int ny = v.ny, e = v.e_s;
    const long long b = (long long)(t0 - 1) * ny + j;
    if constexpr (KIND == 1) {
        // centre column of U (rows t-1, t, t+1), its side columns at row t, per-row differences
        T u0c = U[b], u1c = U[b + ny];
        T u1m = U[b + ny - 1], u1p = U[b + ny + 1];
        T q0 = U[b - 1] - U[b + 1], q1 = u1m - u1p;
#pragma unroll 4
        for (int t = t0; t <= t1; ++t) {
            const long long o = (long long)t * ny + j;
            const T u2m = U[o + ny - 1], u2c = U[o + ny], u2p = U[o + ny + 1];
            const T q2 = u2m - u2p;
            const T mix = q0 - q2;
            T f = ldg(v.S(SL_WG) + o) * mix;
            f += ldg(v.S(SL_WW) + o) * u0c;
            f += ldg(v.S(SL_WS) + o) * u1m;
            f += ldg(v.S(SL_WC) + o) * u1c;
            f += ldg(v.S(SL_WN) + o) * u1p;
            f += ldg(v.S(SL_WE) + o) * u2c;
            y = f - ldg(v.S(SL_LA) + o) * y;
            if (t == e) y -= ldg(v.Yv(Y_CHS) + j) * hi;
            Y[o] = y;
            u0c = u1c; u1c = u2c;
            u1m = u2m; u1p = u2p;
            q0 = q1; q1 = q2;
        }
    } else {
        constexpr bool xt = SCH == LSS_ADI_MODIFIED_CRAIG_SNEYD || SCH == LSS_ADI_HUNDSDORFER_VERWER;
        constexpr bool hv = SCH == LSS_ADI_HUNDSDORFER_VERWER;
        // windows: U centre column, Y1 centre column, Delta = Y2 - U (centre column and, at row t,
        // its side columns), per-row differences of Delta
        T uc0 = U[b], uc1 = U[b + ny];
        T y10 = Y1[b], y11 = Y1[b + ny];
        T d0c = Y2[b] - uc0, d1c = Y2[b + ny] - uc1;
        T d1m = Y2[b + ny - 1] - U[b + ny - 1], d1p = Y2[b + ny + 1] - U[b + ny + 1];
        T q0 = (Y2[b - 1] - U[b - 1]) - (Y2[b + 1] - U[b + 1]), q1 = d1m - d1p;
#pragma unroll 4
        for (int t = t0; t <= t1; ++t) {
            const long long o = (long long)t * ny + j;
            const T uc2 = U[o + ny];
            const T d2m = Y2[o + ny - 1] - U[o + ny - 1];
            const T d2p = Y2[o + ny + 1] - U[o + ny + 1];
            const T q2 = d2m - d2p;
            const T mix = q0 - q2;
            T f, y12 = T(0), d2c = T(0);
            if constexpr (hv || KIND == 2) y12 = Y1[o + ny];
            if constexpr (xt) d2c = Y2[o + ny] - uc2;
            if constexpr (hv) {
                f = ldg(v.S(SL_LA) + o) * y10;
                f += ldg(v.S(SL_S2SC) + o) * y11;
                f += ldg(v.S(SL_S2SE) + o) * y12;
                f += ldg(v.S(SL_S2MZ) + o) * mix;
                f += ldg(v.S(SL_X1) + o) * d0c;
                f += ldg(v.S(SL_X2) + o) * d1c;
                f += ldg(v.S(SL_X3) + o) * d2c;
                f += ldg(v.S(SL_X4) + o) * d1m;
                f += ldg(v.S(SL_X5) + o) * d1p;
            } else {
                f = ldg(v.S(SL_LA) + o) * uc0;
                f += ldg(v.S(SL_S2SC) + o) * uc1;
                f += ldg(v.S(SL_S2SE) + o) * uc2;
                f += ldg(v.S(SL_S2IB) + o) * y11;
                f += ldg(v.S(SL_S2MZ) + o) * mix;
                if constexpr (xt) {
                    f += ldg(v.S(SL_X1) + o) * d0c;
                    f += ldg(v.S(SL_X2) + o) * d1c;
                    f += ldg(v.S(SL_X3) + o) * d2c;
                    f += ldg(v.S(SL_X4) + o) * d1m;
                    f += ldg(v.S(SL_X5) + o) * d1p;
                }
            }
            y = f - ldg(v.S(SL_LA) + o) * y;
            if (t == e) y -= ldg(v.Yv(Y_CHS) + j) * hi;
            Y[o] = y;
            uc0 = uc1; uc1 = uc2;
            y10 = y11; y11 = y12;
            d0c = d1c; d1c = d2c;
            d1m = d2m; d1p = d2p;
            q0 = q1; q1 = q2;
        }
    }
    return y;
}

template <typename T, int KIND, int SCH>
__device__ __forceinline__ void s_stage(const inst_view<T> &v, const T *__restrict__ U, const T *__restrict__ Y1,
                                        const T *__restrict__ Y2, T *__restrict__ Y, int l0, int ls)
{
    const int nx = v.nx, ny = v.ny, e = v.e_s;
    for (int j = 1 + l0; j <= ny - 2; j += ls) {
        const int jj = ldg(v.jmap() + j);
        const T lo = U[jj], hi = U[(long long)(nx - 1) * ny + jj];
        T x = s_line_fwd<T, KIND, SCH>(v, U, Y1, Y2, Y, j, 1, e, lo, hi);
#pragma unroll 4
        for (int t = e - 1; t >= 1; --t) {
            const long long o = (long long)t * ny + j;
            x = Y[o] - ldg(v.S(SL_G) + o) * x;
            Y[o] = x;
        }
        Y[j] = lo;
        Y[(long long)(nx - 1) * ny + j] = hi;
    }
}

// The scheme as a template argument: calls f(std::integral_constant<int, SCH>{}).
template <typename F> __device__ __forceinline__ void with_scheme(int scheme, F &&f)
{
    switch (scheme) {
    case LSS_ADI_DOUGLAS_RACHFORD: f(std::integral_constant<int, LSS_ADI_DOUGLAS_RACHFORD>{}); break;
    case LSS_ADI_CRAIG_SNEYD: f(std::integral_constant<int, LSS_ADI_CRAIG_SNEYD>{}); break;
    case LSS_ADI_MODIFIED_CRAIG_SNEYD: f(std::integral_constant<int, LSS_ADI_MODIFIED_CRAIG_SNEYD>{}); break;
    default: f(std::integral_constant<int, LSS_ADI_HUNDSDORFER_VERWER>{}); break;
    }
}

// v-line sweep: line i reads row i of `in` (t-1, t, t+1) and `inh` (t); tables are [t][i].
// v_line_fwd: right-hand side and forward recurrence over t0..t1 from y = y_{t0-1}.
template <typename T>
__device__ __forceinline__ T v_line_fwd(const inst_view<T> &v, const T *__restrict__ in, const T *__restrict__ inh,
                                        T *__restrict__ out, int i, int t0, int t1, T y, T hi)
{
    const int nx = v.nx, ny = v.ny, e = v.e_v;
    const long long row = (long long)i * ny;
    T a0 = in[row + t0 - 1], a1 = in[row + t0];
#pragma unroll 4
    for (int t = t0; t <= t1; ++t) {
        const long long ot = (long long)t * nx + i;
        const T a2 = in[row + t + 1];
        y = v_point<T>(ldg(v.Vt(VL_LA) + ot), ldg(v.Vt(VL_VC) + ot), ldg(v.Vt(VL_VN) + ot), ldg(v.Vt(VL_IB) + ot), a0,
                       a1, a2, inh[row + t], y);
        if (t == e) y = fma_x(-ldg(v.X(X_CHV) + i), hi, y);
        out[row + t] = y;
        a0 = a1; a1 = a2;
    }
    return y;
}

template <typename T>
__device__ __forceinline__ void v_stage(const inst_view<T> &v, const T *__restrict__ in, const T *__restrict__ inh,
                                        const T *__restrict__ sb0, T *__restrict__ out, int l0, int ls)
{
    const int nx = v.nx, ny = v.ny, e = v.e_v;
    for (int i = 1 + l0; i <= nx - 2; i += ls) {
        const int ii = ldg(v.imap() + i);
        const T lo = sb0[ii];
        const T hi = ldg(v.X(X_VHI) + ii);
        const long long row = (long long)i * ny;
        T x = v_line_fwd<T>(v, in, inh, out, i, 1, e, lo, hi);
#pragma unroll 4
        for (int t = e - 1; t >= 1; --t) {
            x = fma_x(-ldg(v.Vt(VL_G) + (long long)t * nx + i), x, out[row + t]);
            out[row + t] = x;
        }
        out[row] = lo;
        out[row + ny - 1] = hi;
    }
}

// v-line sweep through shared-memory tiles.  The lines of a v sweep are rows of the row-major
// state, so lane r of a warp reading its own row walks memory 8 * ny bytes away from its
// neighbours: every load of the plain sweep touches 32 sectors.  Here the warp's 32 consecutive
// lines (lane r owns line i0 + r) move through a per-warp tile of VT columns: the whole warp loads
// `in` (VT + 2 columns, the window's halo included) and `inh`, and stores `out`, as a few
// contiguous row segments per instruction; each lane then runs its line's recurrence from the
// tile.  The per-line arithmetic is that of v_stage, operation for operation (same bits).
constexpr int VT = 4;
template <typename T> struct vtile {
    T in[32][VT + 3]; // columns t-1 .. t+VT of `in` (odd row stride: conflict-free lane reads)
    T io[32][VT + 1]; // `inh`, overwritten by the recurrence's values, stored to `out`
};

// Copies `cols` columns starting at column c0 of rows i0 .. i0+nrows-1 (row stride ny) between
// global memory and the tile rows 0 .. nrows-1 (row stride W), all 32 lanes of the warp
// cooperating (`lane`: this thread's lane in its warp).
template <int W, int CMAX, bool LOAD, typename T>
__device__ __forceinline__ void vtile_copy(T *tile, const T *src, T *dst, long long i0, int ny, int nrows, int c0,
                                           int cols, int lane)
{
#pragma unroll
    for (int q = 0; q < CMAX; ++q) {
        const int idx = lane + 32 * q, r = idx / CMAX, c = idx % CMAX;
        if (r < nrows && c < cols) {
            const long long g = (i0 + r) * ny + c0 + c;
            if constexpr (LOAD) tile[r * W + c] = src[g];
            else dst[g] = tile[r * W + c];
        }
    }
}

template <typename T>
__device__ __forceinline__ void v_lines_tiled(const inst_view<T> &v, const T *__restrict__ in, const T *__restrict__ inh,
                                              const T *__restrict__ sb0, T *__restrict__ out, int i0, vtile<T> &tl)
{
    const int lane = threadIdx.x & 31; // one-dimensional blocks of whole warps
    const int nx = v.nx, ny = v.ny, e = v.e_v;
    const int i = i0 + lane;
    const bool act = i <= nx - 2;
    const int nrows = min(32, nx - 1 - i0);
    T lo = T(0), hi = T(0), y = T(0);
    if (act) {
        const int ii = ldg(v.imap() + i);
        lo = sb0[ii];
        hi = ldg(v.X(X_VHI) + ii);
        y = lo;
    }
    const T chv = act ? ldg(v.X(X_CHV) + i) : T(0);
    // forward recurrence y_t = f_t - la_t y_{t-1}, tiles left to right
    for (int tb = 1; tb <= e; tb += VT) {
        const int kk = min(VT, e - tb + 1);
        vtile_copy<VT + 3, VT + 2, true>(&tl.in[0][0], in, (T *)nullptr, i0, ny, nrows, tb - 1, kk + 2, lane);
        vtile_copy<VT + 1, VT, true>(&tl.io[0][0], inh, (T *)nullptr, i0, ny, nrows, tb, kk, lane);
        __syncwarp();
        if (act) {
#pragma unroll
            for (int k = 0; k < VT; ++k) {
                if (k < kk) {
                    const int t = tb + k;
                    const long long ot = (long long)t * nx + i;
                    y = v_point<T>(ldg(v.Vt(VL_LA) + ot), ldg(v.Vt(VL_VC) + ot), ldg(v.Vt(VL_VN) + ot),
                                   ldg(v.Vt(VL_IB) + ot), tl.in[lane][k], tl.in[lane][k + 1], tl.in[lane][k + 2],
                                   tl.io[lane][k], y);
                    if (t == e) y = fma_x(-chv, hi, y);
                    tl.io[lane][k] = y;
                }
            }
        }
        __syncwarp();
        vtile_copy<VT + 1, VT, false>(&tl.io[0][0], (const T *)nullptr, out, i0, ny, nrows, tb, kk, lane);
        __syncwarp();
    }
    // back substitution x_t = y_t - g_t x_{t+1} (x_e = y_e), tiles right to left
    T x = y;
    for (int te = e - 1; te >= 1; te -= VT) {
        const int kk = min(VT, te), ts = te - kk + 1;
        vtile_copy<VT + 1, VT, true>(&tl.io[0][0], out, (T *)nullptr, i0, ny, nrows, ts, kk, lane);
        __syncwarp();
        if (act) {
#pragma unroll
            for (int k = VT - 1; k >= 0; --k) {
                if (k < kk) {
                    const int t = ts + k;
                    x = fma_x(-ldg(v.Vt(VL_G) + (long long)t * nx + i), x, tl.io[lane][k]);
                    tl.io[lane][k] = x;
                }
            }
        }
        __syncwarp();
        vtile_copy<VT + 1, VT, false>(&tl.io[0][0], (const T *)nullptr, out, i0, ny, nrows, ts, kk, lane);
        __syncwarp();
    }
    if (act) {
        const long long row = (long long)i * ny;
        out[row] = lo;
        out[row + ny - 1] = hi;
    }
}

// v_stage through the warp tiles: the warp of lane (l0 mod 32) takes lines i0 = 1 + (l0 - lane),
// i0 + ls, ... (ls a multiple of 32, all lanes of a warp in the same work split).
template <typename T>
__device__ __forceinline__ void v_stage_tiled(const inst_view<T> &v, const T *__restrict__ in, const T *__restrict__ inh,
                                              const T *__restrict__ sb0, T *__restrict__ out, int l0, int ls,
                                              vtile<T> &tl)
{
    const int nx = v.nx;
    for (int i0 = 1 + (l0 & ~31); i0 <= nx - 2; i0 += ls) v_lines_tiled<T>(v, in, inh, sb0, out, i0, tl);
}

template <typename T> __device__ __forceinline__ inst_view<T> make_view(const bparams<T> &p, const bdesc &d)
{
    inst_view<T> v;
    v.p = &p;
    v.nx = d.nx;
    v.ny = d.ny;
    v.e_s = d.nx - 2;
    v.e_v = d.ny - 2;
    v.o2 = d.o2;
    v.ox = d.ox;
    v.oy = d.oy;
    return v;
}

// One time step U -> Vn of scheme SCH with stage outputs in Y1, Y2, Y3; ends with a group barrier.
template <typename T, int SCH>
__device__ __forceinline__ void fwd_step(const inst_view<T> &v, const T *U, T *Y1, T *Y2, T *Y3, T *Vn, T *sb0,
                                         double bnc, const grp &g)
{
    const int l0 = g.t, ls = g.n;
    b1_stage<T>(v, U, sb0, bnc, l0, ls);
    s_stage<T, 1, SCH>(v, U, nullptr, nullptr, Y1, l0, ls);
    g.sync();
    if constexpr (SCH == LSS_ADI_DOUGLAS_RACHFORD) {
        v_stage<T>(v, U, Y1, sb0, Vn, l0, ls);
    } else {
        v_stage<T>(v, U, Y1, sb0, Y2, l0, ls);
        g.sync();
        s_stage<T, 2, SCH>(v, U, Y1, Y2, Y3, l0, ls);
        g.sync();
        if constexpr (SCH == LSS_ADI_HUNDSDORFER_VERWER)
            v_stage<T>(v, Y2, Y3, sb0, Vn, l0, ls);
        else
            v_stage<T>(v, U, Y3, sb0, Vn, l0, ls);
    }
    g.sync();
    b2_stage<T>(v, Vn, l0, ls);
    g.sync();
}

// Persistent forward kernel of the instances of scheme SCH: CTAs of 4 warps split into groups
// (the layout word of the CTA), each group pulling instances of its class (warps per instance)
// from the class counter.  Register budget 64 per thread (8 CTAs per SM).
constexpr int BATCH_CTA = 32 * MAX_GROUP_WARPS;

template <typename T, int SCH>
__global__ void __launch_bounds__(BATCH_CTA, 8) k_batch_forward(const __grid_constant__ bparams<T> p)
{
    __shared__ int s_idx[MAX_GROUP_WARPS];
    __shared__ int s_bad[MAX_GROUP_WARPS];
    const grp g = make_grp(p.layout[blockIdx.x]);
    int cls = g.n / 32;
    while (true) {
        if (g.t == 0) s_idx[g.gi] = next_instance(p, cls, -1);
        g.sync();
        const int inst = s_idx[g.gi];
        g.sync();
        if (inst < 0) break;
        const bdesc d = p.desc[inst];
        const inst_view<T> v = make_view(p, d);
        T *U = p.U + d.o2, *Vn = p.V + d.o2, *Y1 = p.Y1 + d.o2, *Y2 = p.Y2 + d.o2, *Y3 = p.Y3 + d.o2;
        T *sb0 = p.B0 + d.ox;
        for (int step = 0; step < d.steps; ++step) {
            fwd_step<T, SCH>(v, U, Y1, Y2, Y3, Vn, sb0, d.bnc, g);
            T *tmp = U;
            U = Vn;
            Vn = tmp;
        }
        // value at (eval_s, eval_v) and a finiteness check of the final surface
        if (g.t == 0) s_bad[g.gi] = 0;
        g.sync();
        const long long n = (long long)d.nx * d.ny;
        int bad = 0;
        for (long long q = g.t; q < n; q += g.n) bad |= !isfinite(static_cast<double>(U[q]));
        if (bad) atomicOr(&s_bad[g.gi], 1);
        g.sync();
        if (g.t == 0) {
            const long long o = (long long)d.i0 * d.ny + d.j0;
            p.values[inst] = d.w00 * static_cast<double>(U[o]) + d.w10 * static_cast<double>(U[o + d.ny]) +
                             d.w01 * static_cast<double>(U[o + 1]) + d.w11 * static_cast<double>(U[o + d.ny + 1]);
            p.status[inst] = s_bad[g.gi];
            p.final_in_v[inst] = d.steps & 1;
        }
        g.sync();
    }
}

#include "adi_adjoint.cuh"

// Forward + adjoint of each instance of scheme SCH by one warp group: forward pass keeping a checkpoint every
// d.ck steps (and the stage values of every step of the last segment), then per segment (last
// first) a forward recomputation that keeps the stage values of every step (not needed for the
// last segment), followed by the adjoint steps of the segment in reverse order.
// Results: value, the 5 parameter sensitivities, the final surface (state U arena) and
// dV/d(initial condition) (state V arena).  A group of w warps works in w consecutive workspace
// slices.  Register budget 96 per thread (5 CTAs of 4 warps per SM): fewer spills than at 80, and
// fewer resident CTAs leave each more workspace, so the plan recomputes fewer steps.
#ifndef LSS_FWDADJ_MIN_CTAS
#define LSS_FWDADJ_MIN_CTAS 5
#endif
template <int SCH>
__global__ void __launch_bounds__(BATCH_CTA, LSS_FWDADJ_MIN_CTAS) k_batch_fwdadj(const __grid_constant__ bparams<double> p)
{
    __shared__ int s_idx[MAX_GROUP_WARPS];
    __shared__ int s_bad[MAX_GROUP_WARPS];
    __shared__ double red[MAX_GROUP_WARPS][5];
    const grp g = make_grp(p.layout[blockIdx.x]);
    const int gw = g.n / 32;
    double *ws = p.ws + (long long)(blockIdx.x * MAX_GROUP_WARPS + g.warp0) * p.ws_per_warp;
    int cls = gw;
    while (true) {
        if (g.t == 0) s_idx[g.gi] = next_instance(p, cls, gw * p.ws_per_warp);
        g.sync();
        const int inst = s_idx[g.gi];
        g.sync();
        if (inst < 0) break;
        const bdesc d = p.desc[inst];
        const inst_view<double> v = make_view(p, d);
        const int nx = d.nx, ny = d.ny;
        const long long n = (long long)nx * ny;
        const int c = d.ck;
        const int nseg = (d.steps + c - 1) / c;
        double *sb0 = p.B0 + d.ox;
        // workspace carve-up
        double *CK = ws;                                  // nseg * n
        double *SEG = CK + (long long)nseg * n;           // (c + 1) * 4 * n
        double *W0 = SEG + (long long)(c + 1) * 4 * n;    // n
        double *W1 = W0 + n;                              // n
        double *UB = W1 + n, *VB = UB + n, *Y1B = VB + n, *Y2B = Y1B + n, *Y3B = Y2B + n, *FB = Y3B + n;
        double *TMP = FB + n;
        double *LV = TMP + n, *LS = LV + nx, *HS = LS + ny;
        auto slot = [&](int m, int a) -> double * { return SEG + ((long long)m * 4 + a) * n; };

        // clear what must start at zero for this instance's shape
        for (long long q = g.t; q < n; q += g.n) {
            FB[q] = 0.0;
            Y1B[q] = 0.0;
            Y3B[q] = 0.0;
            CK[q] = static_cast<double>(p.payoff[d.o2 + q]);
        }
        for (int m = 0; m < c; ++m) {
            double *y2 = slot(m, 2);
            for (int q = g.t; q < ny; q += g.n) {
                y2[q] = 0.0;
                y2[(long long)(nx - 1) * ny + q] = 0.0;
            }
        }
        g.sync();
        // forward pass with checkpoints; the steps of the last segment keep their stage values in
        // the segment slots, so the reverse sweep starts without recomputing that segment
        const double *cur = CK;
        const int n0_last = (nseg - 1) * c;
        for (int step = 0; step < d.steps; ++step) {
            if (step >= n0_last) {
                const int m = step - n0_last;
                fwd_step<double, SCH>(v, cur, slot(m, 1), slot(m, 2), slot(m, 3), slot(m + 1, 0), sb0, d.bnc, g);
                cur = slot(m + 1, 0);
                continue;
            }
            double *next = ((step + 1) % c == 0 && step + 1 < d.steps) ? CK + (long long)((step + 1) / c) * n
                                                                        : ((step & 1) ? W1 : W0);
            fwd_step<double, SCH>(v, cur, slot(0, 1), slot(0, 2), slot(0, 3), next, sb0, d.bnc, g);
            cur = next;
        }
        // value, finiteness, final surface
        if (g.t == 0) s_bad[g.gi] = 0;
        g.sync();
        int bad = 0;
        double *outU = p.U + d.o2;
        for (long long q = g.t; q < n; q += g.n) {
            const double val = cur[q];
            bad |= !isfinite(val);
            outU[q] = val;
            VB[q] = 0.0;
        }
        if (bad) atomicOr(&s_bad[g.gi], 1);
        g.sync();
        if (g.t == 0) {
            const long long o = (long long)d.i0 * ny + d.j0;
            p.values[inst] = d.w00 * cur[o] + d.w10 * cur[o + ny] + d.w01 * cur[o + 1] + d.w11 * cur[o + ny + 1];
            p.status[inst] = s_bad[g.gi];
            p.final_in_v[inst] = 0;
            VB[o] = d.w00;
            VB[o + ny] = d.w10;
            VB[o + 1] = d.w01;
            VB[o + ny + 1] = d.w11;
        }
        g.sync();
        // reverse sweep over the segments
        adj_acc acc;
        for (int q = 0; q < 5; ++q) acc.s[q] = 0.0;
        acc.vk = acc.vt = acc.vs1 = acc.vs2 = acc.vb = 0.0;
        double *ub = UB, *vb = VB;
        for (int sgi = nseg - 1; sgi >= 0; --sgi) {
            const int n0 = sgi * c;
            const int L = min(c, d.steps - n0);
            const double *u0 = CK + (long long)sgi * n;
            for (int m = 0; m < L && sgi < nseg - 1; ++m) {
                const double *um = (m == 0) ? u0 : slot(m, 0);
                fwd_step<double, SCH>(v, um, slot(m, 1), slot(m, 2), slot(m, 3), slot(m + 1, 0), sb0, d.bnc, g);
            }
            for (int m = L - 1; m >= 0; --m) {
                const double *um = (m == 0) ? u0 : slot(m, 0);
                adj_step<SCH>(v, d, um, slot(m, 1), slot(m, 2), slot(m, 3), slot(m + 1, 0), vb, ub, Y1B, Y2B, Y3B, FB,
                              TMP, LV, LS, HS, acc, d.a_tau0 + d.a_dtau * (n0 + m), g);
                double *t = ub;
                ub = vb;
                vb = t;
            }
        }
        // vb = adjoint of the initial condition
        double *outL = p.V + d.o2;
        for (long long q = g.t; q < n; q += g.n) outL[q] = vb[q];
        const double th = d.a_theta, ni = d.a_ni;
        double gr[5];
        // order in the output: kappa, theta, sigma, rho, r
        gr[0] = acc.s[1] + ni * th * acc.vk;
        gr[1] = acc.s[2] + ni * th * acc.vt;
        gr[2] = acc.s[3] + ni * th * acc.vs1 + d.a_betat * th * acc.vs2;
        gr[3] = acc.s[4];
        gr[4] = acc.s[0] + d.a_halfk * th * acc.vb;
        // sum over the group: within each warp by shuffles, then the warps in order
        for (int q = 0; q < 5; ++q)
            for (int off = 16; off > 0; off >>= 1) gr[q] += __shfl_down_sync(0xffffffffu, gr[q], off);
        for (int w = 0; w < gw; ++w) {
            if (g.t == 32 * w)
                for (int q = 0; q < 5; ++q) red[g.gi][q] = (w == 0 ? 0.0 : red[g.gi][q]) + gr[q];
            g.sync();
        }
        if (g.t < 5) p.grads[5LL * inst + g.t] = red[g.gi][g.t];
        g.sync();
    }
}

// ------------------------------------------------------------------------------------------
// wide path: one (large) instance, one kernel per stage over all threads of the grid, same
// stage arithmetic as the batched kernel (bit-identical results for the same instance)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int gstride() { return gridDim.x * blockDim.x; }

template <typename T> __global__ void k_wide_b1(const __grid_constant__ bparams<T> p, const T *U, T *b0)
{
    const bdesc d = p.desc[0];
    const inst_view<T> v = make_view(p, d);
    b1_stage<T>(v, U, b0, d.bnc, gtid(), gstride());
}
template <typename T, int KIND>
__global__ void k_wide_s(const __grid_constant__ bparams<T> p, const T *U, const T *Y1, const T *Y2, T *Y)
{
    const bdesc d = p.desc[0];
    const inst_view<T> v = make_view(p, d);
    with_scheme(d.scheme, [&](auto sch) { s_stage<T, KIND, decltype(sch)::value>(v, U, Y1, Y2, Y, gtid(), gstride()); });
}
// thread-per-line v sweep of the wide path, rows through shared-memory tiles (TILED) or read in
// place; the two give the same bits, the autotuner keeps the faster for the instance
template <typename T, bool TILED>
__global__ void k_wide_v(const __grid_constant__ bparams<T> p, const T *in, const T *inh, const T *b0, T *out)
{
    const bdesc d = p.desc[0];
    const inst_view<T> v = make_view(p, d);
    if constexpr (TILED) {
        __shared__ vtile<T> s_vt[1]; // blocks of one warp
        v_stage_tiled<T>(v, in, inh, b0, out, gtid(), gstride(), s_vt[0]);
    } else {
        v_stage<T>(v, in, inh, b0, out, gtid(), gstride());
    }
}
template <typename T> __global__ void k_wide_b2(const __grid_constant__ bparams<T> p, T *Vn)
{
    const bdesc d = p.desc[0];
    const inst_view<T> v = make_view(p, d);
    b2_stage<T>(v, Vn, gtid(), gstride());
}
// Partitioned line solves of the wide path.  A large single instance has only Nx or Ny
// lines per sweep -- a few warps per SM, far below what the FP64 pipe needs -- so each line
// is cut into P chunks solved concurrently (CTA: L = 8, 16 or 32 lines x P chunks).  Both recurrences
// of the factorised solve are first order and linear:
//   y_t = f_t - la_t y_{t-1}:  y_t = yhat_t + hf_t y_in,  hf_t = prod_{s=t0..t} (-la_s)
//   x_t = y_t - g_t x_{t+1}:   x_t = xhat_t + hb_t x_in,  hb_t = prod_{s=t..t1} (-g_s)
// where yhat / xhat are the chunk-local solutions from a zero start and hf / hb the
// time-invariant chunk products (k_wide_spikes).  A chunk's incoming value is composed
// from the other chunks' end values in shared memory.  Three passes over the chunk: local
// forward solve; forward fix-up fused with the local back substitution; back fix-up.
__device__ __forceinline__ void chunk_range(int e, int P, int c, int &t0, int &t1)
{
    t0 = 1 + static_cast<int>((static_cast<long long>(c) * e) / P);
    t1 = static_cast<int>((static_cast<long long>(c + 1) * e) / P);
}

// The recurrence of the time-dependent S-line factorisation, partitioned like the line solves
// (CTA: L lines x P chunks).  beta_t = b_t - a_t c_{t-1} / beta_{t-1} is the Moebius map of the
// matrix [[b_t, -a_t c_{t-1}], [1, 0]] applied to beta_{t-1}: each chunk forms the product of its
// rows' matrices (rescaled every 8 rows: only the ratio matters), a chunk composes the maps of
// the chunks before it to get its incoming beta, then runs its own rows' recurrence from it
// (1/beta and gamma = c/beta), so the serial chain is a chunk long instead of a line long.
// Same values as the serial recurrence up to the rounding of the incoming beta of each chunk.
template <typename T>
__global__ void __launch_bounds__(1024) k_tdep_s_factor(const double *__restrict__ base, long long n, int nx, int ny,
                                                        double th, T *S0)
{
    __shared__ double sm[4][1024]; // each chunk's map [[m11, m12], [m21, m22]], indexed [c * L + line]
    const int L = blockDim.x, P = blockDim.y, lane = threadIdx.x, c = threadIdx.y;
    const int j = 1 + blockIdx.x * L + lane;
    const bool act = j <= ny - 2;
    const int e = nx - 2, k = c * L + lane;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    const double *__restrict__ bM = base, *__restrict__ bP = base + n, *__restrict__ bZ = base + 2 * n;
    if (act) {
        double m11 = 1.0, m12 = 0.0, m21 = 0.0, m22 = 1.0;
        double pprev = t0 > 1 ? bP[(long long)(t0 - 1) * ny + j] : 0.0; // P of row t-1 (c_{t-1} = -theta P)
        for (int t = t0; t <= t1; ++t) {
            const long long o = (long long)t * ny + j;
            const double b = 1.0 + th * bZ[o];
            const double ac = t > 1 ? (-th * bM[o]) * (-th * pprev) : 0.0; // a_t c_{t-1}
            pprev = bP[o];
            const double n11 = b * m11 - ac * m21, n12 = b * m12 - ac * m22;
            m21 = m11;
            m22 = m12;
            m11 = n11;
            m12 = n12;
            if (((t - t0) & 7) == 7) {
                const double sc = 1.0 / fmax(fabs(m11), fabs(m21));
                m11 *= sc; m12 *= sc; m21 *= sc; m22 *= sc;
            }
        }
        sm[0][k] = m11; sm[1][k] = m12; sm[2][k] = m21; sm[3][k] = m22;
    }
    __syncthreads();
    if (!act) return;
    // beta_{t0-1}: the maps of chunks 0 .. c-1 applied in order (chunk 0 starts at row 1, whose
    // map ignores its argument: a_1 c_0 = 0)
    double x = 1.0;
    for (int q = 0; q < c; ++q) {
        const int kq = q * L + lane;
        x = (sm[0][kq] * x + sm[1][kq]) / (sm[2][kq] * x + sm[3][kq]);
    }
    double gam = t0 > 1 ? (-th * bP[(long long)(t0 - 1) * ny + j]) / x : 0.0;
    for (int t = t0; t <= t1; ++t) {
        const long long o = (long long)t * ny + j;
        const double a = -th * bM[o], b = 1.0 + th * bZ[o], cc = -th * bP[o];
        const double beta = (t == 1) ? b : b - a * gam;
        S0[SL_IB * n + o] = static_cast<T>(1.0 / beta);
        if (t < e) gam = cc / beta;
        S0[SL_G * n + o] = static_cast<T>(t < e ? gam : 0.0);
    }
}

// hf / hb of every chunk of every line; lines along j ([t][j] tables, S) or i ([t][i], v)
template <typename T>
__global__ void k_wide_spikes(const T *__restrict__ la, const T *__restrict__ g, T *__restrict__ hf,
                              T *__restrict__ hb, int lines, int stride, int e, int P)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (lines - 2) * P) return;
    const int l = 1 + q / P, c = q % P;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    T pr = T(1);
    for (int t = t0; t <= t1; ++t) {
        const long long o = (long long)t * stride + l;
        pr *= -la[o];
        hf[o] = pr;
    }
    pr = T(1);
    for (int t = t1; t >= t0; --t) {
        const long long o = (long long)t * stride + l;
        pr *= -g[o];
        hb[o] = pr;
    }
}

template <typename T, int KIND>
__global__ void __launch_bounds__(1024) k_wide_s_chunk(const __grid_constant__ bparams<T> p, const T *U, const T *Y1,
                                                        const T *Y2, T *Y, const T *__restrict__ hf,
                                                        const T *__restrict__ hb)
{
    __shared__ T sa_s[1024], sb_s[1024];
    const carry2d<T> sa{sa_s, static_cast<int>(blockDim.x)}, sb{sb_s, static_cast<int>(blockDim.x)};
    const bdesc d = p.desc[0];
    const inst_view<T> v = make_view(p, d);
    const int nx = d.nx, ny = d.ny, e = nx - 2, P = blockDim.y, c = threadIdx.y, lane = threadIdx.x;
    const int j = 1 + blockIdx.x * blockDim.x + lane;
    const bool act = j <= ny - 2;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    T lo = T(0), hi = T(0);
    if (act) {
        const int jj = ldg(v.jmap() + j);
        lo = U[jj];
        hi = U[(long long)(nx - 1) * ny + jj];
        with_scheme(d.scheme, [&](auto sch) {
            sb[c][lane] = s_line_fwd<T, KIND, decltype(sch)::value>(v, U, Y1, Y2, Y, j, t0, t1, c == 0 ? lo : T(0), hi);
        });
        sa[c][lane] = hf[(long long)t1 * ny + j];
    }
    __syncthreads();
    T xh = T(0);
    if (act) {
        T yin = T(0);
        if (c > 0) {
            yin = sb[0][lane];
            for (int q = 1; q < c; ++q) yin = sb[q][lane] + sa[q][lane] * yin;
        }
        for (int t = t1; t >= t0; --t) {
            const long long o = (long long)t * ny + j;
            const T y = (c > 0) ? Y[o] + hf[o] * yin : Y[o];
            xh = y - ldg(v.S(SL_G) + o) * xh;
            Y[o] = xh;
        }
    }
    __syncthreads();
    if (act) {
        sb[c][lane] = xh;
        sa[c][lane] = hb[(long long)t0 * ny + j];
    }
    __syncthreads();
    if (act) {
        if (c < P - 1) {
            T xin = sb[P - 1][lane];
            for (int q = P - 2; q > c; --q) xin = sb[q][lane] + sa[q][lane] * xin;
            for (int t = t0; t <= t1; ++t) {
                const long long o = (long long)t * ny + j;
                Y[o] += hb[o] * xin;
            }
        }
        if (c == 0) Y[j] = lo;
        if (c == P - 1) Y[(long long)(nx - 1) * ny + j] = hi;
    }
}

// Partitioned v sweep with the rows read in place (see k_wide_s_chunk; same bits as
// k_wide_v_chunk, whose rows go through shared-memory tiles).
template <typename T>
__global__ void __launch_bounds__(1024) k_wide_v_chunk_plain(const __grid_constant__ bparams<T> p, const T *in, const T *inh,
                                                        const T *b0, T *out, const T *__restrict__ hf,
                                                        const T *__restrict__ hb)
{
    __shared__ T sa_s[1024], sb_s[1024];
    const carry2d<T> sa{sa_s, static_cast<int>(blockDim.x)}, sb{sb_s, static_cast<int>(blockDim.x)};
    const bdesc d = p.desc[0];
    const inst_view<T> v = make_view(p, d);
    const int nx = d.nx, ny = d.ny, e = ny - 2, P = blockDim.y, c = threadIdx.y, lane = threadIdx.x;
    const int i = 1 + blockIdx.x * blockDim.x + lane;
    const bool act = i <= nx - 2;
    const long long row = (long long)i * ny;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    T lo = T(0), hi = T(0);
    if (act) {
        const int ii = ldg(v.imap() + i);
        lo = b0[ii];
        hi = ldg(v.X(X_VHI) + ii);
        sb[c][lane] = v_line_fwd<T>(v, in, inh, out, i, t0, t1, c == 0 ? lo : T(0), hi);
        sa[c][lane] = hf[(long long)t1 * nx + i];
    }
    __syncthreads();
    T xh = T(0);
    if (act) {
        T yin = T(0);
        if (c > 0) {
            yin = sb[0][lane];
            for (int q = 1; q < c; ++q) yin = fma_x(sa[q][lane], yin, sb[q][lane]);
        }
        for (int t = t1; t >= t0; --t) {
            const long long ot = (long long)t * nx + i;
            const T y = (c > 0) ? fma_x(hf[ot], yin, out[row + t]) : out[row + t];
            xh = fma_x(-ldg(v.Vt(VL_G) + ot), xh, y);
            out[row + t] = xh;
        }
    }
    __syncthreads();
    if (act) {
        sb[c][lane] = xh;
        sa[c][lane] = hb[(long long)t0 * nx + i];
    }
    __syncthreads();
    if (act) {
        if (c < P - 1) {
            T xin = sb[P - 1][lane];
            for (int q = P - 2; q > c; --q) xin = fma_x(sa[q][lane], xin, sb[q][lane]);
            for (int t = t0; t <= t1; ++t) out[row + t] = fma_x(hb[(long long)t * nx + i], xin, out[row + t]);
        }
        if (c == 0) out[row] = lo;
        if (c == P - 1) out[row + ny - 1] = hi;
    }
}

// Copy between global memory and a warp's tile where each tile row r has its own global offset
// and length: owner(r, off, cnt) gives them (cnt = 0 for rows without work); `lane`: this
// thread's lane in its warp.
template <int W, int CMAX, bool LOAD, typename T, typename F>
__device__ __forceinline__ void vtile_copy_rows(T *tile, const T *src, T *dst, F owner, int lane)
{
#pragma unroll
    for (int q = 0; q < CMAX; ++q) {
        const int idx = lane + 32 * q, r = idx / CMAX, c = idx % CMAX;
        long long off;
        int cnt;
        owner(r, off, cnt);
        if (c < cnt) {
            if constexpr (LOAD) tile[r * W + c] = src[off + c];
            else dst[off + c] = tile[r * W + c];
        }
    }
}

// Partitioned v sweep (see k_wide_s_chunk) with the rows of `in`, `inh` and `out` moved through
// per-warp shared-memory tiles (v_lines_tiled): the CTA's threads are (lines x chunks) with the
// line index fastest, so a warp holds 32 / L chunks of L lines (or one chunk of 32 lines), each
// lane its own line and chunk.  Every tile row is a contiguous segment of one state row; the
// arithmetic per point is that of the thread-per-line recurrences, operation for operation.
// The CTA must be whole warps (L * P a multiple of 32, set_wide_chunks).  Dynamic shared memory:
// one vtile per warp.
template <typename T>
__global__ void __launch_bounds__(1024) k_wide_v_chunk(const __grid_constant__ bparams<T> p, const T *in, const T *inh,
                                                        const T *b0, T *out, const T *__restrict__ hf,
                                                        const T *__restrict__ hb)
{
    __shared__ T sa_s[1024], sb_s[1024];
    const carry2d<T> sa{sa_s, static_cast<int>(blockDim.x)}, sb{sb_s, static_cast<int>(blockDim.x)};
    extern __shared__ unsigned char vt_raw[];
    const bdesc d = p.desc[0];
    const inst_view<T> v = make_view(p, d);
    const int nx = d.nx, ny = d.ny, e = ny - 2, P = blockDim.y, c = threadIdx.y, lane = threadIdx.x, L = blockDim.x;
    const int lin = c * L + lane, w = lin >> 5, wl = lin & 31;
    vtile<T> &tl = reinterpret_cast<vtile<T> *>(vt_raw)[w];
    const int i = 1 + blockIdx.x * L + lane;
    const bool act = i <= nx - 2;
    const long long row = (long long)i * ny;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    // tile row r of this warp: line and chunk of the warp's lane r
    auto line_of = [&](int r, int &ir, int &cr) {
        const int lr = (w << 5) + r;
        cr = lr / L;
        ir = 1 + blockIdx.x * L + lr % L;
    };
    const int steps = (t1 - t0 + VT) / VT; // tiles of this lane's chunk
    int steps_max = steps;
    for (int off = 16; off > 0; off >>= 1) steps_max = max(steps_max, __shfl_xor_sync(0xffffffffu, steps_max, off));
    T lo = T(0), hi = T(0);
    if (act) {
        const int ii = ldg(v.imap() + i);
        lo = b0[ii];
        hi = ldg(v.X(X_VHI) + ii);
    }
    const T chv = act ? ldg(v.X(X_CHV) + i) : T(0);
    // pass 1: local forward recurrence of the chunk (from lo on chunk 0, from 0 on the others)
    T y = c == 0 ? lo : T(0);
    for (int jt = 0; jt < steps_max; ++jt) {
        auto own_in = [&](int r, long long &off, int &cnt) {
            int ir, cr, a, b;
            line_of(r, ir, cr);
            chunk_range(e, P, cr, a, b);
            const int tb = a + jt * VT, kk = min(VT, b - tb + 1);
            cnt = (ir <= nx - 2 && kk > 0) ? kk + 2 : 0;
            off = (long long)ir * ny + tb - 1;
        };
        auto own_h = [&](int r, long long &off, int &cnt) {
            int ir, cr, a, b;
            line_of(r, ir, cr);
            chunk_range(e, P, cr, a, b);
            const int tb = a + jt * VT, kk = min(VT, b - tb + 1);
            cnt = (ir <= nx - 2 && kk > 0) ? kk : 0;
            off = (long long)ir * ny + tb;
        };
        vtile_copy_rows<VT + 3, VT + 2, true>(&tl.in[0][0], in, (T *)nullptr, own_in, wl);
        vtile_copy_rows<VT + 1, VT, true>(&tl.io[0][0], inh, (T *)nullptr, own_h, wl);
        __syncwarp();
        const int tb = t0 + jt * VT, kk = min(VT, t1 - tb + 1);
        if (act) {
#pragma unroll
            for (int k = 0; k < VT; ++k) {
                if (k < kk) {
                    const int t = tb + k;
                    const long long ot = (long long)t * nx + i;
                    y = v_point<T>(ldg(v.Vt(VL_LA) + ot), ldg(v.Vt(VL_VC) + ot), ldg(v.Vt(VL_VN) + ot),
                                   ldg(v.Vt(VL_IB) + ot), tl.in[wl][k], tl.in[wl][k + 1], tl.in[wl][k + 2],
                                   tl.io[wl][k], y);
                    if (t == e) y = fma_x(-chv, hi, y);
                    tl.io[wl][k] = y;
                }
            }
        }
        __syncwarp();
        vtile_copy_rows<VT + 1, VT, false>(&tl.io[0][0], (const T *)nullptr, out, own_h, wl);
        __syncwarp();
    }
    if (act) {
        sb[c][lane] = y;
        sa[c][lane] = hf[(long long)t1 * nx + i];
    }
    __syncthreads();
    // pass 2: forward fix-up y += hf yin with the incoming value composed from the chunks before,
    // fused with the chunk's back substitution from a zero start
    T yin = T(0);
    if (act && c > 0) {
        yin = sb[0][lane];
        for (int q = 1; q < c; ++q) yin = fma_x(sa[q][lane], yin, sb[q][lane]);
    }
    T xh = T(0);
    for (int jt = 0; jt < steps_max; ++jt) {
        // tiles from the chunk's end: columns [b - (jt+1) VT + 1, b - jt VT] clipped to the chunk
        auto own_b = [&](int r, long long &off, int &cnt) {
            int ir, cr, a, b;
            line_of(r, ir, cr);
            chunk_range(e, P, cr, a, b);
            const int te = b - jt * VT, ts = max(a, te - VT + 1);
            cnt = (ir <= nx - 2 && te >= a) ? te - ts + 1 : 0;
            off = (long long)ir * ny + ts;
        };
        vtile_copy_rows<VT + 1, VT, true>(&tl.io[0][0], out, (T *)nullptr, own_b, wl);
        __syncwarp();
        const int te = t1 - jt * VT, ts = max(t0, te - VT + 1);
        if (act && te >= t0) {
#pragma unroll
            for (int k = VT - 1; k >= 0; --k) {
                if (k <= te - ts) {
                    const int t = ts + k;
                    const long long ot = (long long)t * nx + i;
                    const T yv = (c > 0) ? fma_x(hf[ot], yin, tl.io[wl][k]) : tl.io[wl][k];
                    xh = fma_x(-ldg(v.Vt(VL_G) + ot), xh, yv);
                    tl.io[wl][k] = xh;
                }
            }
        }
        __syncwarp();
        vtile_copy_rows<VT + 1, VT, false>(&tl.io[0][0], (const T *)nullptr, out, own_b, wl);
        __syncwarp();
    }
    __syncthreads();
    if (act) {
        sb[c][lane] = xh;
        sa[c][lane] = hb[(long long)t0 * nx + i];
    }
    __syncthreads();
    // pass 3: backward fix-up x += hb xin (all chunks but the last)
    T xin = T(0);
    if (act && c < P - 1) {
        xin = sb[P - 1][lane];
        for (int q = P - 2; q > c; --q) xin = fma_x(sa[q][lane], xin, sb[q][lane]);
    }
    for (int jt = 0; jt < steps_max; ++jt) {
        auto own_f = [&](int r, long long &off, int &cnt) {
            int ir, cr, a, b;
            line_of(r, ir, cr);
            chunk_range(e, P, cr, a, b);
            const int tb = a + jt * VT, kk = min(VT, b - tb + 1);
            cnt = (ir <= nx - 2 && kk > 0 && cr < P - 1) ? kk : 0;
            off = (long long)ir * ny + tb;
        };
        vtile_copy_rows<VT + 1, VT, true>(&tl.io[0][0], out, (T *)nullptr, own_f, wl);
        __syncwarp();
        const int tb = t0 + jt * VT, kk = min(VT, t1 - tb + 1);
        if (act && c < P - 1) {
#pragma unroll
            for (int k = 0; k < VT; ++k)
                if (k < kk) tl.io[wl][k] = fma_x(hb[(long long)(tb + k) * nx + i], xin, tl.io[wl][k]);
        }
        __syncwarp();
        vtile_copy_rows<VT + 1, VT, false>(&tl.io[0][0], (const T *)nullptr, out, own_f, wl);
        __syncwarp();
    }
    if (act) {
        if (c == 0) out[row] = lo;
        if (c == P - 1) out[row + ny - 1] = hi;
    }
}

// ------------------------------------------------------------------------------------------
// wide forward + adjoint of one large FP64 instance: the adjoint stages of adi_adjoint.cuh as
// one kernel each over all threads (thread per line / column), host-sequenced like the
// forward; each thread's parameter sums live in `acc` (structure of arrays, 10 x nthr) between
// kernels and are reduced once at the end.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void acc_load(adj_acc &acc, const double *a, long long nthr, long long t)
{
    for (int q = 0; q < 5; ++q) acc.s[q] = a[q * nthr + t];
    acc.vk = a[5 * nthr + t];
    acc.vt = a[6 * nthr + t];
    acc.vs1 = a[7 * nthr + t];
    acc.vs2 = a[8 * nthr + t];
    acc.vb = a[9 * nthr + t];
}
__device__ __forceinline__ void acc_store(const adj_acc &acc, double *a, long long nthr, long long t)
{
    for (int q = 0; q < 5; ++q) a[q * nthr + t] = acc.s[q];
    a[5 * nthr + t] = acc.vk;
    a[6 * nthr + t] = acc.vt;
    a[7 * nthr + t] = acc.vs1;
    a[8 * nthr + t] = acc.vs2;
    a[9 * nthr + t] = acc.vb;
}

__global__ void k_wadj_b2(const __grid_constant__ bparams<double> p, double *VB, double *UB)
{
    const bdesc d = p.desc[0];
    const inst_view<double> v = make_view(p, d);
    adj_b2(v, VB, UB, d.scheme == LSS_ADI_HUNDSDORFER_VERWER, gtid(), gstride());
}

template <bool FIRST>
__global__ void k_wadj_v(const __grid_constant__ bparams<double> p, const double *in, const double *out, const double *XB,
                         double *INB, double *INHB, double *TMP, double *LV, double *acc_a, long long nacc)
{
    const bdesc d = p.desc[0];
    const inst_view<double> v = make_view(p, d);
    const long long t = gtid();
    adj_acc acc;
    acc_load(acc, acc_a, nacc, t);
    adj_v<FIRST>(v, in, out, XB, INB, INHB, TMP, LV, acc, gtid(), gstride());
    acc_store(acc, acc_a, nacc, t);
}

template <int KIND>
__global__ void k_wadj_s(const __grid_constant__ bparams<double> p, const double *U, const double *Y1, const double *Y2,
                         const double *Yo, const double *XB, double *FB, double *TMP, double *LS, double *HS, double *UB,
                         double *Y1B, double *acc_a, long long nacc, double tau)
{
    const bdesc d = p.desc[0];
    const inst_view<double> v = make_view(p, d);
    const long long t = gtid();
    adj_acc acc;
    acc_load(acc, acc_a, nacc, t);
    with_scheme(d.scheme, [&](auto sch) {
        adj_s<KIND, decltype(sch)::value>(v, d, U, Y1, Y2, Yo, XB, FB, TMP, LS, HS, UB, Y1B, acc, tau, gtid(), gstride());
    });
    acc_store(acc, acc_a, nacc, t);
}

// Partitioned adjoint line solves (the wide adjoint's counterpart of k_wide_s_chunk /
// k_wide_v_chunk): the transposed factorised solve
//   z_t = xbar_t - g_{t-1} z_{t-1}  (t = 1..e),   w_t = z_t - la_{t+1} w_{t+1}  (t = e..1)
// is cut into chunks with the chunk products hz_t = prod_{s=t0..t} (-g_{s-1}) and
// hw_t = prod_{s=t..t1} (-la_{s+1}); after the final w of the whole line is in TMP, each chunk
// applies the point-local terms (right-hand-side adjoints, parameter sums).
template <typename T>
__global__ void k_wadj_spikes(const T *__restrict__ la, const T *__restrict__ g, T *__restrict__ hz,
                              T *__restrict__ hw, int lines, int stride, int e, int P)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (lines - 2) * P) return;
    const int l = 1 + q / P, c = q % P;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    T pr = T(1);
    for (int t = t0; t <= t1; ++t) {
        pr *= (t > 1) ? -g[(long long)(t - 1) * stride + l] : T(0);
        hz[(long long)t * stride + l] = pr;
    }
    pr = T(1);
    for (int t = t1; t >= t0; --t) {
        pr *= (t < e) ? -la[(long long)(t + 1) * stride + l] : T(0);
        hw[(long long)t * stride + l] = pr;
    }
}

// z and w of one chunk of a line: element t of the line at base[t * st] in TMP, tables at
// tab + t * ts; carries through the block's shared arrays (rows: chunks, columns: lines).
__device__ __forceinline__ void adj_chunk_solve(double *__restrict__ TMP, long long base, long long st,
                                                const double *__restrict__ XB, const double *__restrict__ G,
                                                const double *__restrict__ LA, const double *__restrict__ hz,
                                                const double *__restrict__ hw, long long tab, long long ts, int e,
                                                int t0, int t1, int c, int P, int lane, bool act,
                                                const carry2d<double> &sa, const carry2d<double> &sb)
{
    double z = 0.0;
    if (act) {
        for (int t = t0; t <= t1; ++t) {
            const double gprev = (t > 1) ? __ldg(G + tab + (long long)(t - 1) * ts) : 0.0;
            z = XB[base + t * st] - gprev * z;
            TMP[base + t * st] = z;
        }
        sb[c][lane] = z;
        sa[c][lane] = hz[tab + (long long)t1 * ts];
    }
    __syncthreads();
    double w = 0.0;
    if (act) {
        double zin = 0.0;
        if (c > 0) {
            zin = sb[0][lane];
            for (int q = 1; q < c; ++q) zin = sb[q][lane] + sa[q][lane] * zin;
        }
        double la_next = 0.0;
        for (int t = t1; t >= t0; --t) {
            const double zt = (c > 0) ? TMP[base + t * st] + hz[tab + (long long)t * ts] * zin : TMP[base + t * st];
            w = zt - la_next * w;
            TMP[base + t * st] = w;
            la_next = __ldg(LA + tab + (long long)t * ts);
        }
    }
    __syncthreads();
    if (act) {
        sb[c][lane] = w;
        sa[c][lane] = hw[tab + (long long)t0 * ts];
    }
    __syncthreads();
    if (act && c < P - 1) {
        double win = sb[P - 1][lane];
        for (int q = P - 2; q > c; --q) win = sb[q][lane] + sa[q][lane] * win;
        for (int t = t0; t <= t1; ++t) TMP[base + t * st] += hw[tab + (long long)t * ts] * win;
    }
    __syncthreads();
}

template <bool FIRST>
__global__ void __launch_bounds__(1024) k_wadj_v_chunk(const __grid_constant__ bparams<double> p, const double *in,
                                                        const double *out, const double *XB, double *INB, double *INHB,
                                                        double *TMP, double *LV, double *acc_a, long long nacc,
                                                        const double *__restrict__ hz, const double *__restrict__ hw)
{
    __shared__ double sa_s[1024], sb_s[1024];
    const carry2d<double> sa{sa_s, static_cast<int>(blockDim.x)}, sb{sb_s, static_cast<int>(blockDim.x)};
    const bdesc d = p.desc[0];
    const inst_view<double> v = make_view(p, d);
    const int nx = d.nx, ny = d.ny, e = ny - 2, P = blockDim.y, c = threadIdx.y, lane = threadIdx.x;
    const int i = 1 + blockIdx.x * blockDim.x + lane;
    const bool act = i <= nx - 2;
    const long long row = (long long)i * ny, tid = ((long long)blockIdx.x * P + c) * blockDim.x + lane;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    adj_chunk_solve(TMP, row, 1, XB, v.Vt(VL_G), v.Vt(VL_LA), hz, hw, i, nx, e, t0, t1, c, P, lane, act, sa, sb);
    if (!act) return;
    adj_acc acc;
    acc_load(acc, acc_a, nacc, tid);
    const double *LA = v.Vt(VL_LA), *VC = v.Vt(VL_VC), *VN = v.Vt(VL_VN), *IB = v.Vt(VL_IB);
    for (int t = t1; t >= t0; --t) {
        const long long ot = (long long)t * nx + i;
        const double w0 = TMP[row + t];
        const double w1 = (t + 1 <= e) ? TMP[row + t + 1] : 0.0, w2 = (t + 2 <= e) ? TMP[row + t + 2] : 0.0;
        const double la2 = (t + 2 <= e) ? __ldg(LA + ot + 2LL * nx) : 0.0, vc1 = (t + 1 <= e) ? __ldg(VC + ot + nx) : 0.0;
        const double fin = la2 * w2 + vc1 * w1 + __ldg(VN + ot) * w0; // adjoint of in(t+1)
        if (FIRST) INB[row + t + 1] = fin; else INB[row + t + 1] += fin;
        const double mu = __ldg(IB + ot) * w0;
        if (FIRST) INHB[row + t] = mu; else INHB[row + t] += mu;
        adj_v_sum(v, t, mu, in[row + t - 1] - out[row + t - 1], in[row + t] - out[row + t],
                  in[row + t + 1] - out[row + t + 1], acc);
    }
    if (c == 0) {
        const double w1 = TMP[row + 1], w2 = (2 <= e) ? TMP[row + 2] : 0.0;
        const double la1 = __ldg(LA + nx + i), la2 = (2 <= e) ? __ldg(LA + 2LL * nx + i) : 0.0;
        const double a1 = la2 * w2 + __ldg(VC + nx + i) * w1, a0 = la1 * w1;
        if (FIRST) { INB[row + 1] = a1; INB[row] = a0; }
        else { INB[row + 1] += a1; INB[row] += a0; }
        const double lob = -la1 * w1 + XB[row];
        if (FIRST) LV[i] = lob; else LV[i] += lob;
    }
    acc_store(acc, acc_a, nacc, tid);
}

template <int KIND>
__global__ void __launch_bounds__(1024) k_wadj_s_chunk(const __grid_constant__ bparams<double> p, const double *U,
                                                        const double *Y1, const double *Y2, const double *Yo,
                                                        const double *XB, double *FB, double *TMP, double *LS, double *HS,
                                                        double *UB, double *Y1B, double *acc_a, long long nacc, double tau,
                                                        const double *__restrict__ hz, const double *__restrict__ hw)
{
    __shared__ double sa_s[1024], sb_s[1024];
    const carry2d<double> sa{sa_s, static_cast<int>(blockDim.x)}, sb{sb_s, static_cast<int>(blockDim.x)};
    const bdesc d = p.desc[0];
    const inst_view<double> v = make_view(p, d);
    const int nx = d.nx, ny = d.ny, e = nx - 2, P = blockDim.y, c = threadIdx.y, lane = threadIdx.x;
    const int j = 1 + blockIdx.x * blockDim.x + lane;
    const bool act = j <= ny - 2;
    const long long tid = ((long long)blockIdx.x * P + c) * blockDim.x + lane;
    int t0, t1;
    chunk_range(e, P, c, t0, t1);
    adj_chunk_solve(TMP, j, ny, XB, v.S(SL_G), v.S(SL_LA), hz, hw, j, ny, e, t0, t1, c, P, lane, act, sa, sb);
    if (!act) return;
    const bool sabr = d.model == LSS_ADI_SABR;
    const double th = d.a_theta, omth = 1.0 - d.a_theta;
    adj_acc acc;
    acc_load(acc, acc_a, nacc, tid);
    const double *LA = v.S(SL_LA), *IB = v.S(SL_IB);
    with_scheme(d.scheme, [&](auto sch) {
        constexpr int SCH = decltype(sch)::value;
        constexpr bool hv = SCH == LSS_ADI_HUNDSDORFER_VERWER;
        s_sums ps = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        // three-row window over the chunk's rows (adj_s_row / adj_s_point)
        s_row rh = adj_s_row<KIND, SCH>(U, Y1, Y2, Yo, (long long)(t1 + 1) * ny + j, th, omth);
        s_row rc = adj_s_row<KIND, SCH>(U, Y1, Y2, Yo, (long long)t1 * ny + j, th, omth);
        for (int t = t1; t >= t0; --t) {
            const long long o = (long long)t * ny + j;
            const s_row rl = adj_s_row<KIND, SCH>(U, Y1, Y2, Yo, o - ny, th, omth);
            const double w0 = TMP[o];
            FB[o] = w0;
            const double mu = __ldg(IB + o) * w0;
            if constexpr (KIND == 2) {
                const double w1 = (t + 1 <= e) ? TMP[o + ny] : 0.0, w2 = (t + 2 <= e) ? TMP[o + 2LL * ny] : 0.0;
                const double la2 = (t + 2 <= e) ? __ldg(LA + o + 2LL * ny) : 0.0;
                const double sc1 = (t + 1 <= e) ? __ldg(v.S(SL_S2SC) + o + ny) : 0.0;
                const double fin = la2 * w2 + sc1 * w1 + __ldg(v.S(SL_S2SE) + o) * w0;
                if constexpr (hv) {
                    Y1B[o + ny] = fin;
                } else {
                    UB[o + ny] += fin;
                    Y1B[o] = mu;
                }
            }
            const double muX = mu * __ldg(v.X(X_HX) + t);
            const double muC = sabr ? mu * __ldg(v.X(X_HC) + t) : muX;
            adj_s_point<KIND, SCH>(v, ps, rh, rc, rl, mu, muX, muC, t, sabr);
            rh = rc;
            rc = rl;
        }
        if (c == 0) {
            const double w1 = TMP[(long long)ny + j], la1 = __ldg(LA + ny + j);
            LS[j] = -la1 * w1 + XB[j];
            if constexpr (KIND == 2) {
                const double w2 = (2 <= e) ? TMP[2LL * ny + j] : 0.0, la2 = (2 <= e) ? __ldg(LA + 2LL * ny + j) : 0.0;
                const double a1 = la2 * w2 + __ldg(v.S(SL_S2SC) + ny + j) * w1, a0 = la1 * w1;
                if constexpr (hv) {
                    Y1B[(long long)ny + j] = a1;
                    Y1B[j] = a0;
                } else {
                    UB[(long long)ny + j] += a1;
                    UB[j] += a0;
                }
            }
        }
        if (c == P - 1) HS[j] = -__ldg(v.Yv(Y_CHS) + j) * TMP[(long long)e * ny + j] + XB[(long long)(nx - 1) * ny + j];
        adj_s_line<KIND, SCH>(v, d, j, ps, tau, sabr, acc);
    });
    acc_store(acc, acc_a, nacc, tid);
}

// Gather with one thread per grid point; the B1 parameter sums of column 0 go to acc slot p.
template <int KIND>
__global__ void k_wadj_gather2d(const __grid_constant__ bparams<double> p, const double *U, const double *FB,
                                const double *LS, const double *HS, const double *LV, double *UB, double *Y2B,
                                double *acc_a, long long nacc, double tau)
{
    const bdesc d = p.desc[0];
    const inst_view<double> v = make_view(p, d);
    const long long n = (long long)d.nx * d.ny;
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int pr = static_cast<int>(o / d.ny), q = static_cast<int>(o % d.ny);
    double lsum = 0.0, hsum = 0.0;
    if (pr == 0 || pr == d.nx - 1) adj_line_ends(v, LS, HS, q, lsum, hsum);
    adj_acc acc;
    if (q == 0) {
        acc_load(acc, acc_a, nacc, pr);
    } else {
        for (int k = 0; k < 5; ++k) acc.s[k] = 0.0;
        acc.vk = acc.vt = acc.vs1 = acc.vs2 = acc.vb = 0.0;
    }
    adj_gather_point<KIND>(v, d, U, FB, LV, UB, Y2B, acc, tau, pr, q, lsum, hsum);
    if (q == 0) acc_store(acc, acc_a, nacc, pr);
}

// final surface out, adjoint arrays cleared, finiteness of the final surface
__global__ void k_wadj_begin(const __grid_constant__ bparams<double> p, const double *cur, double *VB, double *FB,
                             double *Y1B, double *Y3B)
{
    const bdesc d = p.desc[0];
    const long long n = (long long)d.nx * d.ny;
    int bad = 0;
    for (long long q = gtid(); q < n; q += gstride()) {
        const double val = cur[q];
        bad |= !isfinite(val);
        p.U[q] = val;
        VB[q] = 0.0;
        FB[q] = 0.0;
        Y1B[q] = 0.0;
        Y3B[q] = 0.0;
    }
    if (bad) atomicOr(p.status, 1);
}
// value and its bilinear weights as the adjoint seed
__global__ void k_wadj_seed(const __grid_constant__ bparams<double> p, const double *cur, double *VB)
{
    const bdesc d = p.desc[0];
    const long long o = (long long)d.i0 * d.ny + d.j0;
    p.values[0] = d.w00 * cur[o] + d.w10 * cur[o + d.ny] + d.w01 * cur[o + 1] + d.w11 * cur[o + d.ny + 1];
    p.final_in_v[0] = 0;
    VB[o] = d.w00;
    VB[o + d.ny] = d.w10;
    VB[o + 1] = d.w01;
    VB[o + d.ny + 1] = d.w11;
}
// sum of the per-thread parameter sums; output order kappa, theta, sigma, rho, r
__global__ void __launch_bounds__(256) k_wadj_reduce(const __grid_constant__ bparams<double> p, const double *acc_a,
                                                     long long nthr)
{
    __shared__ double red[10][256];
    for (int q = 0; q < 10; ++q) {
        double sum = 0.0;
        for (long long t = threadIdx.x; t < nthr; t += 256) sum += acc_a[q * nthr + t];
        red[q][threadIdx.x] = sum;
    }
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int q = 0; q < 10; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const bdesc d = p.desc[0];
        const double th = d.a_theta, ni = d.a_ni;
        p.grads[0] = red[1][0] + ni * th * red[5][0];
        p.grads[1] = red[2][0] + ni * th * red[6][0];
        p.grads[2] = red[3][0] + ni * th * red[7][0] + d.a_betat * th * red[8][0];
        p.grads[3] = red[4][0];
        p.grads[4] = red[0][0] + d.a_halfk * th * red[9][0];
    }
}

// value, finiteness flag and final-array flag of the single instance
// value at the evaluation point and finiteness of the final surface, grid-wide (the status word
// is cleared before the time loop; any block that sees a non-finite point sets it)
template <typename T> __global__ void k_wide_finish(const __grid_constant__ bparams<T> p, const T *U)
{
    const bdesc d = p.desc[0];
    const long long n = (long long)d.nx * d.ny;
    int b = 0;
    for (long long q = gtid(); q < n; q += gstride()) b |= !isfinite(static_cast<double>(U[q]));
    b = __syncthreads_or(b);
    if (b && threadIdx.x == 0) atomicOr(p.status, 1);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const long long o = (long long)d.i0 * d.ny + d.j0;
        p.values[0] = d.w00 * static_cast<double>(U[o]) + d.w10 * static_cast<double>(U[o + d.ny]) +
                      d.w01 * static_cast<double>(U[o + 1]) + d.w11 * static_cast<double>(U[o + d.ny + 1]);
        p.final_in_v[0] = d.steps & 1;
    }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
template <typename T> struct batch_typed {
    int count = 0;
    std::vector<bdesc> desc;
    std::vector<int> order;
    std::vector<long long> gps;
    long long total_n = 0, total_x = 0, total_y = 0;
    dbuf<bdesc> d_desc;
    dbuf<int> d_order, d_counter, d_status, d_final, d_imap, d_jmap;
    dbuf<double> d_values;
    dbuf<T> state, stab, vtab, xarena, yarena;
    std::vector<std::vector<T>> payoff_host;
    dbuf<T> d_payoff; // concatenated initial conditions (sum n)
    long long launches = 0;
    // forward + adjoint
    bool adjoint_ok = false;      // FP64, Heston and SABR with r = 0
    std::string adjoint_why;
    int ck_override = 0;          // checkpoint interval (0 = planned from the workspace cap)
    double ws_cap = 0.0;          // adjoint workspace cap in bytes (0 = a quarter of the device memory)
    dbuf<double> d_grads, d_ws;
    dbuf<T> b0arena;              // nx arena: boundary column of the step (persistent kernels)
    // warp-group plan of a persistent kernel (per mode): instance classes, class queues, CTA
    // layouts and, for mode 1, the workspace slices and checkpoint intervals
    // (one launch per scheme present: each specialisation gets its own register allocation)
    struct group_plan {
        int grid = 0;
        int start[MAX_GROUP_WARPS + 1] = {}, cnt[MAX_GROUP_WARPS + 1] = {};
        long long need[MAX_GROUP_WARPS + 1] = {};
        std::vector<int> order, layout;
        dbuf<int> d_order, d_layout;
    };
    static constexpr int NSCHEMES = 4; // LSS_ADI_DOUGLAS_RACHFORD .. LSS_ADI_HUNDSDORFER_VERWER
    struct mode_plan {
        bool valid = false;
        int gcap = 0, override_ck = -1;
        double cap = -1.0;
        long long per_warp = 0;
        group_plan sch[NSCHEMES];
    } plan[2];
    int sms = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_mode = -1;

    ~batch_typed()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (wide_graph) cudaGraphExecDestroy(wide_graph);
    }

    bparams<T> params()
    {
        bparams<T> p{};
        p.desc = d_desc.p;
        p.order = d_order.p;
        p.count = count;
        p.counter = d_counter.p;
        p.B0 = b0arena.p;
        p.U = state.p;
        p.V = state.p + total_n;
        p.Y1 = state.p + 2 * total_n;
        p.Y2 = state.p + 3 * total_n;
        p.Y3 = state.p + 4 * total_n;
        for (int s = 0; s < SL_COUNT; ++s) p.S[s] = stab.p + s * total_n;
        for (int s = 0; s < VL_COUNT; ++s) p.Vt[s] = vtab.p + s * total_n;
        for (int s = 0; s < X_COUNT; ++s) p.X[s] = xarena.p + s * total_x;
        for (int s = 0; s < Y_COUNT; ++s) p.Yv[s] = yarena.p + s * total_y;
        p.imap = d_imap.p;
        p.jmap = d_jmap.p;
        p.values = d_values.p;
        p.status = d_status.p;
        p.final_in_v = d_final.p;
        p.grads = d_grads.p;
        p.ws = d_ws.p;
        p.payoff = d_payoff.p;
        return p;
    }
    // params() with the class queues and layouts of mode m's plan for scheme sc
    bparams<T> params_for(int m, int sc)
    {
        bparams<T> p = params();
        const group_plan &g = plan[m].sch[sc];
        p.order = g.d_order.p;
        p.layout = g.d_layout.p;
        p.counter = d_counter.p + sc * (MAX_GROUP_WARPS + 1);
        for (int c = 0; c <= MAX_GROUP_WARPS; ++c) {
            p.cls_start[c] = g.start[c];
            p.cls_count[c] = g.cnt[c];
            p.cls_need[c] = g.need[c];
        }
        p.ws_per_warp = plan[m].per_warp;
        return p;
    }

    int create(const lss_adi_problem *ps, int n);
    int prepare_adjoint(cudaStream_t s);
    double ws_bytes_allowed();
    // most threads per instance (32 x warps of a group) of the persistent kernels, per mode;
    // chosen by autotune()
    int bs_mode[2] = {BATCH_CTA, BATCH_CTA};
    int make_plan(int mode); // (re)plans mode's groups when its inputs changed
    int launch_forward(cudaStream_t s);
    int launch_fwdadj(cudaStream_t s);
    int autotune(int mode, int *chosen, cudaStream_t s);
    // wide path (count == 1)
    dbuf<T> d_b0;
    cudaGraphExec_t wide_graph = nullptr;
    int wide_ps = 1, wide_pv = 1;   // chunks per S line / per v line (1: thread per line)
    int wide_ls = 32, wide_lv = 32; // lines per CTA of the partitioned kernels (CTA: lines x chunks)
    bool wide_vtile = true;         // v sweeps move their rows through shared-memory tiles (same bits)
    dbuf<T> d_spk;                  // chunk products: S hf, S hb, v hf, v hb (n each)
    int set_wide_chunks(int ps, int pv, cudaStream_t s, int ls = 0, int lv = 0); // ls, lv 0: by SM count
    int autotune_wide(cudaStream_t s);
    template <int KIND> void launch_wide_s(cudaStream_t s, const bparams<T> &p, const T *U, const T *Y1, const T *Y2, T *Y);
    void launch_wide_v(cudaStream_t s, const bparams<T> &p, const T *in, const T *inh, const T *b0, T *out);
    void enqueue_wide_step(cudaStream_t s, const bparams<T> &p, const T *U, T *Y1, T *Y2, T *Y3, T *V);
    int enqueue_wide(cudaStream_t s);
    int run_wide(cudaStream_t s, bool use_graph);
    // wide forward + adjoint (count == 1, FP64)
    dbuf<double> d_wws;
    long long wws_need = 0;
    dbuf<T> d_aspk;                 // adjoint chunk products: S hz, S hw, v hz, v hw (n each)
    int aspk_ps = 0, aspk_pv = 0;
    int enqueue_wide_adjoint(cudaStream_t s);
    // time-dependent coefficients (SABR with r != 0; one FP64 instance on the wide kernels):
    // before each step, forward or adjoint, the S-line tables are rebuilt at the step's time
    bool tdep = false;
    dbuf<double> td_buf;            // base tables (7 n), a_static, c_static, ab (n each), per_i (5 nx), xs (3 nx)
    tdep_params td{};
    std::vector<double> td_da, td_dc; // D(t)^(2(1-beta)), D(t)^(1-beta) per step
    double td_theta = 0.0, td_zeta = 0.0, td_gamma = 0.0;
    int init_tdep(const lss_adi_problem &p);
    // products: 1 = the forward chunk products of the S lines, 2 = the adjoint's
    void refresh_step(cudaStream_t s, int step, int products);
    int enqueue(int mode, cudaStream_t s);
    int run(int mode, cudaStream_t s, bool use_graph);
};

template <typename T> int batch_typed<T>::create(const lss_adi_problem *ps, int n)
{
    count = n;
    desc.resize(n);
    gps.resize(n);
    long long on = 0, ox = 0, oy = 0;
    for (int k = 0; k < n; ++k) {
        desc[k].nx = ps[k].nx;
        desc[k].ny = ps[k].ny;
        desc[k].steps = ps[k].nt - 1;
        desc[k].scheme = ps[k].scheme;
        desc[k].o2 = on;
        desc[k].ox = static_cast<int>(ox);
        desc[k].oy = static_cast<int>(oy);
        gps[k] = static_cast<long long>(ps[k].nx) * ps[k].ny * (ps[k].nt - 1);
        on += static_cast<long long>(ps[k].nx) * ps[k].ny;
        ox += ps[k].nx;
        oy += ps[k].ny;
    }
    total_n = on;
    total_x = ox;
    total_y = oy;
    if (ox > (1LL << 31) || oy > (1LL << 31)) return set_error(LSS_ADI_EINVAL, "batch too large");

    // host tables in the reference arithmetic, in parallel over instances
    std::vector<double> base(7 * static_cast<size_t>(total_n));
    std::vector<T> xh(X_COUNT * static_cast<size_t>(total_x)), yh(Y_COUNT * static_cast<size_t>(total_y));
    std::vector<int> imh(total_x), jmh(total_y);
    std::vector<double> scal(3 * static_cast<size_t>(n));
    std::vector<T> pay(static_cast<size_t>(total_n));
    const unsigned nthr = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    std::vector<int> errs(nthr, 0);
    for (unsigned w = 0; w < nthr; ++w) {
        pool.emplace_back([&, w]() {
            try {
                for (int k = static_cast<int>(w); k < n; k += static_cast<int>(nthr)) {
                    instance_tables<T> tt;
                    build_tables_for<T>(ps[k], tt);
                    const bdesc &d = desc[k];
                    const size_t nn = static_cast<size_t>(d.nx) * d.ny;
                    for (int s = 0; s < 7; ++s)
                        for (size_t q = 0; q < nn; ++q)
                            base[s * static_cast<size_t>(total_n) + d.o2 + q] = static_cast<double>(tt.coef[s * nn + q]);
                    std::copy(tt.payoff.begin(), tt.payoff.end(), pay.begin() + d.o2);
                    const double th = tt.sc.theta, ni = tt.sc.ni, dl = tt.sc.delta, rk = tt.sc.rho;
                    scal[3 * k] = th;
                    scal[3 * k + 1] = static_cast<double>(tt.sc.zeta);
                    scal[3 * k + 2] = static_cast<double>(tt.sc.gamma);
                    for (int i = 0; i < d.nx; ++i) {
                        const double D = tt.coef_v0[i], E = tt.coef_v0[d.nx + i], F = tt.coef_v0[2 * d.nx + i];
                        xh[XB_M * total_x + d.ox + i] = static_cast<T>(-dl * D);
                        xh[XB_C * total_x + d.ox + i] = static_cast<T>(1.0 - 3.0 * ni * E + rk * F);
                        xh[XB_P * total_x + d.ox + i] = static_cast<T>(dl * D);
                        xh[XB_2 * total_x + d.ox + i] = static_cast<T>(-ni * E);
                        xh[XB_1 * total_x + d.ox + i] = static_cast<T>(4.0 * ni * E);
                        xh[X_VHI * total_x + d.ox + i] = tt.v_hi[i];
                        imh[d.ox + i] = tt.imap[i];
                    }
                    const double h1 = tt.sc.h1;
                    {
                        // coefficient derivatives (adjoint), double.  Heston: a = vS^2/2, b = sigma^2 v/2,
                        // c = rho sigma v S, d = rS, e = kappa (theta - v), f = -r.  SABR (r = 0, D = 1):
                        // a = v^2 F^(2 beta) D^(2(1-beta))/2, b = nu^2 v^2/2, c = rho nu v^2 F^beta D^(1-beta),
                        // d = rF, e = 0, f = -r (sigma carries nu).
                        sinh_map<double> g;
                        g.init(ps[k]);
                        const double sg = ps[k].sigma, bt = ps[k].sabr_beta;
                        const bool sabr = ps[k].model == LSS_ADI_SABR;
                        for (int i = 0; i < d.nx; ++i) {
                            const double z = static_cast<double>(tt.sc.h1) * i;
                            const double x = g.x(z), A = g.a_der(z), Add = g.c_der(z);
                            xh[X_HX * total_x + d.ox + i] = static_cast<T>(x / A);
                            xh[X_HC * total_x + d.ox + i] = static_cast<T>(sabr ? std::pow(x, bt) / A : x / A);
                            xh[X_HA * total_x + d.ox + i] = static_cast<T>(sabr ? std::pow(x, 2.0 * bt) / (A * A) : 0.0);
                            xh[X_HDD * total_x + d.ox + i] = static_cast<T>(sabr ? std::pow(x, 2.0 * bt) * Add / (A * A * A) : 0.0);
                        }
                        for (int j = 0; j < d.ny; ++j) {
                            const double e = static_cast<double>(tt.sc.h2) * j;
                            const double B = g.b_der(e), Bdd = g.d_der(e), vv = g.y(e);
                            const double vb = sabr ? vv * vv : vv; // the v factor of b and c
                            yh[Y_HY * total_y + d.oy + j] = static_cast<T>(vb / B);
                            yh[Y_BS * total_y + d.oy + j] = static_cast<T>(sg * vb / (B * B));
                            yh[Y_EK * total_y + d.oy + j] = static_cast<T>(sabr ? 0.0 : (ps[k].theta_v - vv) / B);
                            yh[Y_ET * total_y + d.oy + j] = static_cast<T>(sabr ? 0.0 : ps[k].kappa / B);
                            yh[Y_ES * total_y + d.oy + j] = static_cast<T>(-sg * vb * Bdd / (B * B * B));
                            yh[Y_HV2 * total_y + d.oy + j] = static_cast<T>(sabr ? 0.5 * vv * vv : 0.0);
                        }
                        desc[k].model = ps[k].model;
                        desc[k].a_alphat = static_cast<double>(tt.sc.alpha);
                        desc[k].a_omb = 1.0 - bt;
                        const double kk = static_cast<double>(tt.sc.k);
                        desc[k].a_tau0 = ps[k].forward ? ps[k].maturity - kk : kk;
                        desc[k].a_dtau = ps[k].forward ? -kk : kk;
                        desc[k].a_delta = static_cast<double>(tt.sc.delta);
                        desc[k].a_halfk = 0.5 * static_cast<double>(tt.sc.k);
                        desc[k].a_ni = static_cast<double>(tt.sc.ni);
                        desc[k].a_betat = static_cast<double>(tt.sc.beta);
                        desc[k].a_sigma = sg;
                        desc[k].a_rho = ps[k].rho;
                        desc[k].a_theta = static_cast<double>(tt.sc.theta);
                        desc[k].a_zeta = static_cast<double>(tt.sc.zeta);
                        desc[k].a_gamma = static_cast<double>(tt.sc.gamma);
                        desc[k].a_k = static_cast<double>(tt.sc.k);
                        desc[k].ck = std::max(1, static_cast<int>(std::ceil(std::sqrt(static_cast<double>(d.steps)))));
                    }
                    for (int j = 0; j < d.ny; ++j) {
                        yh[Y_SLO * total_y + d.oy + j] = tt.s_lo[j];
                        yh[Y_B2C * total_y + d.oy + j] = static_cast<T>(2.0 * h1 * static_cast<double>(tt.s_hi_neu[j]) / 3.0);
                        jmh[d.oy + j] = tt.jmap[j];
                    }
                    // modified Craig-Sneyd with zeta == theta adds (zeta - theta) * (...) = 0: it is
                    // Craig-Sneyd (the reference's surfaces are bit-identical), so run the CS stencil
                    if (ps[k].scheme == LSS_ADI_MODIFIED_CRAIG_SNEYD && tt.sc.zeta == tt.sc.theta)
                        desc[k].scheme = LSS_ADI_CRAIG_SNEYD;
                    const double DN = tt.coef_v0[d.nx - 1];
                    desc[k].bnc = -dl * (2.0 * h1 * static_cast<double>(tt.s_hi_neu[0])) * DN;
                    const bilinear b = make_bilinear(tt.x.data(), d.nx, tt.y.data(), d.ny, ps[k].eval_s, ps[k].eval_v);
                    desc[k].i0 = b.i0;
                    desc[k].j0 = b.j0;
                    desc[k].w00 = b.w00;
                    desc[k].w10 = b.w10;
                    desc[k].w01 = b.w01;
                    desc[k].w11 = b.w11;
                }
            } catch (...) {
                errs[w] = 1;
            }
        });
    }
    for (auto &t : pool) t.join();
    for (int e : errs)
        if (e) return set_error(LSS_ADI_ENOMEM, "batch: host table construction failed");

    // longest instances first
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return gps[a] > gps[b]; });

    LSS_CUDA_TRY(d_desc.alloc(n), "batch: allocating descriptors");
    LSS_CUDA_TRY(d_desc.upload(desc.data(), n), "batch: uploading descriptors");
    LSS_CUDA_TRY(d_order.alloc(n), "batch: allocating order");
    LSS_CUDA_TRY(d_order.upload(order.data(), n), "batch: uploading order");
    LSS_CUDA_TRY(d_counter.alloc(4 * (MAX_GROUP_WARPS + 1)), "batch: allocating counters");
    LSS_CUDA_TRY(b0arena.alloc(total_x), "batch: allocating boundary columns");
    LSS_CUDA_TRY(d_status.alloc(n), "batch: allocating status");
    LSS_CUDA_TRY(d_final.alloc(n), "batch: allocating flags");
    LSS_CUDA_TRY(d_values.alloc(n), "batch: allocating values");
    LSS_CUDA_TRY(d_imap.alloc(total_x), "batch: allocating remaps");
    LSS_CUDA_TRY(d_imap.upload(imh.data(), total_x), "batch: uploading remaps");
    LSS_CUDA_TRY(d_jmap.alloc(total_y), "batch: allocating remaps");
    LSS_CUDA_TRY(d_jmap.upload(jmh.data(), total_y), "batch: uploading remaps");
    LSS_CUDA_TRY(xarena.alloc(X_COUNT * total_x), "batch: allocating S boundary arrays");
    LSS_CUDA_TRY(yarena.alloc(Y_COUNT * total_y), "batch: allocating v boundary arrays");
    LSS_CUDA_TRY(state.alloc(5 * total_n), "batch: allocating state");
    LSS_CUDA_TRY(cudaMemset(state.p, 0, state.n * sizeof(T)), "batch: clearing state");
    LSS_CUDA_TRY(d_payoff.alloc(total_n), "batch: allocating initial conditions");
    LSS_CUDA_TRY(d_payoff.upload(pay.data(), total_n), "batch: uploading initial conditions");
    LSS_CUDA_TRY(stab.alloc(SL_COUNT * total_n), "batch: allocating S-line tables");
    LSS_CUDA_TRY(vtab.alloc(VL_COUNT * total_n), "batch: allocating v-line tables");
    // boundary rows/columns of the line tables are read (as zeros) by the adjoint's gather
    LSS_CUDA_TRY(cudaMemset(stab.p, 0, stab.n * sizeof(T)), "batch: clearing S-line tables");
    LSS_CUDA_TRY(cudaMemset(vtab.p, 0, vtab.n * sizeof(T)), "batch: clearing v-line tables");
    LSS_CUDA_TRY(d_grads.alloc(5 * static_cast<size_t>(n)), "batch: allocating gradients");
    LSS_CUDA_TRY(cudaMemset(d_grads.p, 0, d_grads.n * sizeof(double)), "batch: clearing gradients");
    adjoint_ok = std::is_same<T, double>::value;
    adjoint_why = adjoint_ok ? "" : "the adjoint is FP64 only";
    for (int k = 0; k < n && adjoint_ok; ++k) {
        // time-dependent tables are rebuilt per step by the host-sequenced wide kernels only
        if (time_dependent(ps[k]) && n > 1) {
            adjoint_ok = false;
            adjoint_why = "SABR with r != 0 (time-dependent coefficients) runs as a single instance only";
        }
    }

    // factorise on the device from the base tables
    {
        dbuf<double> d_base, d_scal;
        dbuf<long long> d_ls;
        dbuf<bdesc> dd;
        LSS_CUDA_TRY(d_base.alloc(base.size()), "batch: allocating base tables");
        LSS_CUDA_TRY(d_base.upload(base.data(), base.size()), "batch: uploading base tables");
        LSS_CUDA_TRY(d_scal.alloc(scal.size()), "batch: allocating scalars");
        LSS_CUDA_TRY(d_scal.upload(scal.data(), scal.size()), "batch: uploading scalars");
        LSS_CUDA_TRY(cudaMemcpy(xarena.p, xh.data(), xh.size() * sizeof(T), cudaMemcpyHostToDevice), "batch: x arena");
        LSS_CUDA_TRY(cudaMemcpy(yarena.p, yh.data(), yh.size() * sizeof(T), cudaMemcpyHostToDevice), "batch: y arena");
        LSS_CUDA_TRY(d_ls.alloc(n), "batch: line offsets");
        setup_params sp{};
        sp.desc = d_desc.p;
        sp.count = n;
        sp.base = d_base.p;
        sp.total_n = total_n;
        sp.scal = d_scal.p;
        sp.line_start = d_ls.p;
        // S lines: ny - 2 per instance
        std::vector<long long> ls(n);
        long long acc = 0;
        for (int k = 0; k < n; ++k) { ls[k] = acc; acc += desc[k].ny - 2; }
        LSS_CUDA_TRY(d_ls.upload(ls.data(), n), "batch: line offsets");
        sp.total_lines = acc;
        k_setup_s_lines<T><<<grid_for(acc, 128), 128>>>(sp, stab.p, total_n, yarena.p + Y_CHS * total_y);
        LSS_CUDA_TRY(cudaGetLastError(), "batch: launching S-line set-up");
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "batch: S-line set-up");
        acc = 0;
        for (int k = 0; k < n; ++k) { ls[k] = acc; acc += desc[k].nx - 2; }
        LSS_CUDA_TRY(d_ls.upload(ls.data(), n), "batch: line offsets");
        sp.total_lines = acc;
        k_setup_v_lines<T><<<grid_for(acc, 128), 128>>>(sp, vtab.p, total_n, xarena.p + X_CHV * total_x);
        LSS_CUDA_TRY(cudaGetLastError(), "batch: launching v-line set-up");
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "batch: v-line set-up");
    }
    int dev = 0, sms = 0; // local
    LSS_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    LSS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    this->sms = sms;
    if (n == 1) LSS_CUDA_TRY(d_b0.alloc(desc[0].nx), "batch: allocating the boundary column");
    if (n == 1 && time_dependent(ps[0])) return init_tdep(ps[0]);
    return LSS_ADI_OK;
}

// Device copies of the time-independent factors of a time-dependent instance (FP64 only).
template <typename T> int batch_typed<T>::init_tdep(const lss_adi_problem &p)
{
    if (!std::is_same<T, double>::value)
        return set_error(LSS_ADI_EUNSUPPORTED, "batch: time-dependent coefficients on the wide kernels are FP64 only");
    instance_tables<double> tt;
    build_tables<double>(p, tt);
    const bdesc &d = desc[0];
    const long long n = total_n;
    const int nx = d.nx;
    const size_t off_stat = 7 * static_cast<size_t>(n), off_pi = off_stat + 3 * static_cast<size_t>(n),
                 off_xs = off_pi + 5 * static_cast<size_t>(nx), total = off_xs + 3 * static_cast<size_t>(nx);
    std::vector<double> h(total, 0.0);
    std::copy(tt.coef.begin(), tt.coef.end(), h.begin());
    std::copy(tt.a_static.begin(), tt.a_static.end(), h.begin() + off_stat);
    std::copy(tt.c_static.begin(), tt.c_static.end(), h.begin() + off_stat + n);
    std::copy(tt.ab.begin(), tt.ab.end(), h.begin() + off_stat + 2 * n);
    std::copy(tt.per_i.begin(), tt.per_i.end(), h.begin() + off_pi);
    // the adjoint's S-factors at D = 1 (the arena holds them as built by create)
    std::vector<T> xa(X_COUNT * static_cast<size_t>(total_x));
    LSS_CUDA_TRY(cudaMemcpy(xa.data(), xarena.p, xa.size() * sizeof(T), cudaMemcpyDeviceToHost), "batch: x arena");
    for (int i = 0; i < nx; ++i) {
        h[off_xs + i] = static_cast<double>(xa[X_HA * total_x + i]);
        h[off_xs + nx + i] = static_cast<double>(xa[X_HDD * total_x + i]);
        h[off_xs + 2 * nx + i] = static_cast<double>(xa[X_HC * total_x + i]);
    }
    LSS_CUDA_TRY(td_buf.alloc(total), "batch: allocating time-dependent tables");
    LSS_CUDA_TRY(td_buf.upload(h.data(), total), "batch: uploading time-dependent tables");
    td_theta = tt.sc.theta;
    td_zeta = tt.sc.zeta;
    td_gamma = tt.sc.gamma;
    LSS_CUDA_TRY(cudaDeviceSynchronize(), "batch: time-dependent tables");
    td.base = td_buf.p;
    td.a_static = td_buf.p + off_stat;
    td.c_static = td_buf.p + off_stat + n;
    td.ab = td_buf.p + off_stat + 2 * n;
    td.per_i = td_buf.p + off_pi;
    td.xs = td_buf.p + off_xs;
    td.n = n;
    td.nx = nx;
    td.ny = d.ny;
    td.alpha = tt.sc.alpha;
    td.delta = tt.sc.delta;
    td.two_alpha = tt.two_alpha;
    td.half_rho_f = tt.half_rho_f;
    td_da = tt.step_da;
    td_dc = tt.step_dc;
    tdep = true;
    return LSS_ADI_OK;
}

// The S-line tables (and with `products` the chunk products of the partitioned solves) of
// step `step` of a time-dependent instance, enqueued on s before that step's kernels.
template <typename T> void batch_typed<T>::refresh_step(cudaStream_t s, int step, int products)
{
    const bdesc &d = desc[0];
    const long long n = total_n;
    k_tdep_refresh<T><<<grid_for(n, 256), 256, 0, s>>>(td, td_da[step], td_dc[step], xarena.p, total_x);
    {
        // chunks of at least 4 rows, at most 32; 8 lines per CTA
        int P = 1;
        while (P < 32 && d.nx - 2 >= 8 * P) P *= 2;
        k_tdep_s_factor<T><<<grid_for(d.ny - 2, 8), dim3(8, P), 0, s>>>(td.base, n, d.nx, d.ny, td_theta, stab.p);
    }
    k_tdep_s_slots<T><<<grid_for(static_cast<long long>(d.nx - 2) * (d.ny - 2), 256), 256, 0, s>>>(
        td.base, n, d.nx, d.ny, d.scheme, td_theta, td_zeta, td_gamma, stab.p, yarena.p + Y_CHS * total_y);
    if (wide_ps > 1) {
        const bparams<T> p = params();
        const int g = grid_for(static_cast<long long>(d.ny - 2) * wide_ps, 128);
        if (products & 1)
            k_wide_spikes<T><<<g, 128, 0, s>>>(p.S[SL_LA], p.S[SL_G], d_spk.p, d_spk.p + n, d.ny, d.ny, d.nx - 2, wide_ps);
        if (products & 2)
            k_wadj_spikes<T><<<g, 128, 0, s>>>(p.S[SL_LA], p.S[SL_G], d_aspk.p, d_aspk.p + n, d.ny, d.ny, d.nx - 2, wide_ps);
    }
}

template <typename T> int batch_typed<T>::prepare_adjoint(cudaStream_t s)
{
    (void)s;
    if (!adjoint_ok) return set_error(LSS_ADI_EUNSUPPORTED, "batch: " + adjoint_why);
    return make_plan(1);
}

// Workspace (doubles) of one instance checkpointed every c steps: nseg checkpoints, the stage
// values of one segment (4 arrays per step plus the segment's end), two scratch states, seven
// adjoint arrays and three line-end vectors.
static long long adj_ws_need(const bdesc &d, int c)
{
    const long long nn = static_cast<long long>(d.nx) * d.ny;
    const long long nseg = (d.steps + c - 1) / c;
    return (nseg + 4LL * (c + 1) + 2 + 7) * nn + d.nx + 2LL * d.ny;
}

// Bytes the adjoint workspace may take: the cap set by lss_adi_batch_set_workspace, by default
// a quarter of the device memory, and never more than half of what is free (counting the
// workspace already held, which a new plan replaces).
template <typename T> double batch_typed<T>::ws_bytes_allowed()
{
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return ws_cap > 0.0 ? ws_cap : 0.0;
    }
    // the default (a quarter of the device) leaves at least half of what is free to the caller;
    // a cap the caller sets is honoured up to 90 % of what is free
    const double held = d_ws.p ? static_cast<double>(d_ws.n) * sizeof(double) : 0.0;
    const double avail = static_cast<double>(free_b) + held;
    if (ws_cap > 0.0) return std::min(ws_cap, 0.9 * avail);
    return std::min(0.25 * static_cast<double>(total_b), 0.5 * avail);
}

// CTA layouts (warp-group sizes, one hex digit per group) for `grid` CTAs of MAX_GROUP_WARPS
// warps: each CTA in turn takes the layout that covers the most of the classes' remaining
// shares of the warps (class c's share: its grid-point-steps over all, times the warps); the
// groups' stealing of smaller instances evens out what the rounding leaves.
static std::vector<int> plan_layouts(int grid, const double work[MAX_GROUP_WARPS + 1], int gcap)
{
    struct lay { int code; int w[MAX_GROUP_WARPS + 1]; };
    const lay all[] = {{0x4, {0, 0, 0, 0, 1}}, {0x13, {0, 1, 0, 1, 0}}, {0x22, {0, 0, 2, 0, 0}},
                       {0x112, {0, 2, 1, 0, 0}}, {0x1111, {0, 4, 0, 0, 0}}};
    std::vector<lay> cand;
    for (const lay &l : all) {
        bool ok = true;
        for (int c = gcap + 1; c <= MAX_GROUP_WARPS; ++c) ok = ok && l.w[c] == 0;
        if (ok) cand.push_back(l);
    }
    double tot = 0.0;
    for (int c = 1; c <= MAX_GROUP_WARPS; ++c) tot += work[c];
    double want[MAX_GROUP_WARPS + 1] = {};
    for (int c = 1; c <= MAX_GROUP_WARPS; ++c)
        want[c] = tot > 0.0 ? work[c] / tot * MAX_GROUP_WARPS * grid : 0.0;
    // the first CTA holds a group as large as the largest class that has work, so that every
    // class has a group able to take its instances
    int top = 0;
    for (int c = 1; c <= MAX_GROUP_WARPS; ++c)
        if (work[c] > 0.0) top = c;
    std::vector<int> out(grid);
    for (int b = 0; b < grid; ++b) {
        int best = 0;
        double best_score = -1.0;
        if (b == 0 && top > 0) {
            for (size_t q = 0; q < cand.size(); ++q) {
                bool fits = cand[q].w[top] > 0;
                for (int c = top + 1; c <= MAX_GROUP_WARPS; ++c) fits = fits && cand[q].w[c] == 0;
                if (fits) { best = static_cast<int>(q); break; }
            }
            out[b] = cand[best].code;
            for (int c = 1; c <= MAX_GROUP_WARPS; ++c) want[c] -= cand[best].w[c] * c;
            continue;
        }
        for (size_t q = 0; q < cand.size(); ++q) {
            double score = 0.0;
            for (int c = 1; c <= MAX_GROUP_WARPS; ++c)
                score += std::min(static_cast<double>(cand[q].w[c] * c), std::max(0.0, want[c]));
            if (score > best_score + 1e-9) { best_score = score; best = static_cast<int>(q); }
        }
        out[b] = cand[best].code;
        for (int c = 1; c <= MAX_GROUP_WARPS; ++c) want[c] -= cand[best].w[c] * c;
    }
    return out;
}

// Warp-group plan of mode `mode`: class (warps per instance) of every instance -- one warp per 32
// S lines, at most bs_mode/32 -- and, per scheme present (one launch each), the class queues
// longest first and the CTA layouts; for mode 1 the workspace slices (per warp, within the cap,
// shared by the schemes' launches) and every instance's checkpoint interval: at least
// ceil(sqrt(steps)) (or the fixed interval), else the longest whose workspace fits the slices of
// its class's group.  A cap too small for the minimal slices of every resident CTA runs fewer CTAs.
template <typename T> int batch_typed<T>::make_plan(int mode)
{
    mode_plan &mp = plan[mode];
    const int gcap = std::max(1, std::min(MAX_GROUP_WARPS, bs_mode[mode] / 32));
    if (mp.valid && mp.gcap == gcap && (mode == 0 || (mp.override_ck == ck_override && mp.cap == ws_cap))) return LSS_ADI_OK;
    if (graph && graph_mode == mode) { // a captured launch holds the old plan
        cudaGraphExecDestroy(graph);
        graph = nullptr;
        graph_mode = -1;
    }
    mp.valid = false;
    std::vector<int> cls(count);
    double work[NSCHEMES][MAX_GROUP_WARPS + 1] = {};
    int warps_wanted[NSCHEMES] = {};
    for (int k = 0; k < count; ++k) {
        const int nx = desc[k].nx, ny = desc[k].ny, sc = desc[k].scheme;
        cls[k] = std::max(1, std::min(gcap, (ny - 2 + 31) / 32));
        // the group's threads that have a line, over its threads, per S / v sweep: the class's
        // warps are shared out by work over that efficiency
        const int th = 32 * cls[k];
        const double lines = static_cast<double>(nx - 2) * (ny - 2);
        const double slots = static_cast<double>(nx - 2) * ((ny - 2 + th - 1) / th) * th +
                             static_cast<double>(ny - 2) * ((nx - 2 + th - 1) / th) * th;
        work[sc][cls[k]] += static_cast<double>(gps[k]) * slots / (2.0 * lines);
        warps_wanted[sc] += cls[k];
    }
    int per_sm = 0;
    if constexpr (std::is_same<T, double>::value) {
        if (mode == 1)
            LSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_fwdadj<LSS_ADI_CRAIG_SNEYD>, BATCH_CTA, 0),
                         "occupancy");
    }
    if (mode == 0)
        LSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_forward<T, LSS_ADI_CRAIG_SNEYD>, BATCH_CTA, 0),
                     "occupancy");
    const int resident = sms * std::max(1, per_sm);
    int grid[NSCHEMES];
    for (int sc = 0; sc < NSCHEMES; ++sc)
        grid[sc] = std::max(1, std::min(resident, (warps_wanted[sc] + MAX_GROUP_WARPS - 1) / MAX_GROUP_WARPS));
    mp.per_warp = 0;
    for (int sc = 0; sc < NSCHEMES; ++sc)
        for (int c = 0; c <= MAX_GROUP_WARPS; ++c) mp.sch[sc].need[c] = 0;
    if (mode == 1) {
        std::vector<int> c0(count);
        long long base_w = 1, full_w = 1; // doubles per warp: minimal and no-recomputation slices
        for (int k = 0; k < count; ++k) {
            const bdesc &d = desc[k];
            c0[k] = ck_override > 0 ? std::min(ck_override, d.steps)
                                    : std::max(1, static_cast<int>(std::ceil(std::sqrt(static_cast<double>(d.steps)))));
            base_w = std::max(base_w, (adj_ws_need(d, c0[k]) + cls[k] - 1) / cls[k]);
            full_w = std::max(full_w, (adj_ws_need(d, d.steps) + cls[k] - 1) / cls[k]);
        }
        base_w = (base_w + 31) / 32 * 32;
        const double allowed = ws_bytes_allowed() / sizeof(double);
        const long long fit = static_cast<long long>(allowed / (static_cast<double>(base_w) * MAX_GROUP_WARPS));
        if (fit < 1)
            return set_error(LSS_ADI_ENOMEM, "batch: the adjoint workspace cap (" + std::to_string(allowed * 8.0 / 1e6) +
                                                 " MB) does not hold the checkpoints of the largest instance");
        int gmax = 1;
        for (int sc = 0; sc < NSCHEMES; ++sc) {
            grid[sc] = static_cast<int>(std::min<long long>(grid[sc], fit));
            gmax = std::max(gmax, grid[sc]);
        }
        long long per_warp = base_w;
        if (ck_override <= 0)
            per_warp = std::max(base_w, std::min((full_w + 31) / 32 * 32,
                                                 static_cast<long long>(allowed / (static_cast<double>(gmax) * MAX_GROUP_WARPS)) / 32 * 32));
        bool changed = false;
        for (int k = 0; k < count; ++k) {
            bdesc &d = desc[k];
            int c = c0[k];
            if (ck_override <= 0)
                for (int cc = d.steps; cc > c0[k]; --cc)
                    if (adj_ws_need(d, cc) <= per_warp * cls[k]) { c = cc; break; }
            if (c != d.ck) { d.ck = c; changed = true; }
            long long &nd = mp.sch[d.scheme].need[cls[k]];
            nd = std::max(nd, adj_ws_need(d, c));
        }
        if (changed)
            LSS_CUDA_TRY(cudaMemcpy(d_desc.p, desc.data(), count * sizeof(bdesc), cudaMemcpyHostToDevice), "batch: descriptors");
        mp.per_warp = per_warp;
        const size_t want = static_cast<size_t>(per_warp) * MAX_GROUP_WARPS * gmax;
        if (d_ws.n != want) {
            d_ws.release();
            LSS_CUDA_TRY(d_ws.alloc(want), "batch: allocating adjoint workspace");
        }
    }
    for (int sc = 0; sc < NSCHEMES; ++sc) {
        group_plan &g = mp.sch[sc];
        // class queues, longest first within a class
        g.order.clear();
        for (int c = 0; c <= MAX_GROUP_WARPS; ++c) g.start[c] = g.cnt[c] = 0;
        for (int c = 1; c <= MAX_GROUP_WARPS; ++c) {
            g.start[c] = static_cast<int>(g.order.size());
            for (int k : order)
                if (cls[k] == c && desc[k].scheme == sc) g.order.push_back(k);
            g.cnt[c] = static_cast<int>(g.order.size()) - g.start[c];
        }
        g.grid = g.order.empty() ? 0 : grid[sc];
        if (!g.grid) continue;
        g.layout = plan_layouts(g.grid, work[sc], gcap);
        LSS_CUDA_TRY(g.d_order.alloc(g.order.size()), "batch: allocating class queues");
        LSS_CUDA_TRY(g.d_order.upload(g.order.data(), g.order.size()), "batch: uploading class queues");
        LSS_CUDA_TRY(g.d_layout.alloc(g.grid), "batch: allocating CTA layouts");
        LSS_CUDA_TRY(g.d_layout.upload(g.layout.data(), g.grid), "batch: uploading CTA layouts");
    }
    LSS_CUDA_TRY(cudaDeviceSynchronize(), "batch: plan upload");
    mp.gcap = gcap;
    mp.override_ck = ck_override;
    mp.cap = ws_cap;
    mp.valid = true;
    return LSS_ADI_OK;
}

template <typename T> int batch_typed<T>::launch_forward(cudaStream_t s)
{
    for (int sc = 0; sc < NSCHEMES; ++sc) {
        const group_plan &g = plan[0].sch[sc];
        if (!g.grid) continue;
        const bparams<T> p = params_for(0, sc);
        switch (sc) {
        case LSS_ADI_DOUGLAS_RACHFORD: k_batch_forward<T, LSS_ADI_DOUGLAS_RACHFORD><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
        case LSS_ADI_CRAIG_SNEYD: k_batch_forward<T, LSS_ADI_CRAIG_SNEYD><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
        case LSS_ADI_MODIFIED_CRAIG_SNEYD: k_batch_forward<T, LSS_ADI_MODIFIED_CRAIG_SNEYD><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
        default: k_batch_forward<T, LSS_ADI_HUNDSDORFER_VERWER><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
        }
        LSS_CUDA_TRY(cudaGetLastError(), "batch: launching k_batch_forward");
        ++launches;
    }
    return LSS_ADI_OK;
}

template <typename T> int batch_typed<T>::launch_fwdadj(cudaStream_t s)
{
    if constexpr (std::is_same<T, double>::value) {
        for (int sc = 0; sc < NSCHEMES; ++sc) {
            const group_plan &g = plan[1].sch[sc];
            if (!g.grid) continue;
            const bparams<double> p = params_for(1, sc);
            switch (sc) {
            case LSS_ADI_DOUGLAS_RACHFORD: k_batch_fwdadj<LSS_ADI_DOUGLAS_RACHFORD><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
            case LSS_ADI_CRAIG_SNEYD: k_batch_fwdadj<LSS_ADI_CRAIG_SNEYD><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
            case LSS_ADI_MODIFIED_CRAIG_SNEYD: k_batch_fwdadj<LSS_ADI_MODIFIED_CRAIG_SNEYD><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
            default: k_batch_fwdadj<LSS_ADI_HUNDSDORFER_VERWER><<<g.grid, BATCH_CTA, 0, s>>>(p); break;
            }
            LSS_CUDA_TRY(cudaGetLastError(), "batch: launching k_batch_fwdadj");
            ++launches;
        }
        return LSS_ADI_OK;
    } else {
        (void)s;
        return set_error(LSS_ADI_EUNSUPPORTED, "batch: the adjoint is FP64 only");
    }
}

template <typename T> int batch_typed<T>::enqueue(int mode, cudaStream_t s)
{
    int rc = make_plan(mode == 1 ? 1 : 0);
    if (rc) return rc;
    LSS_CUDA_TRY(cudaMemsetAsync(d_counter.p, 0, d_counter.n * sizeof(int), s), "batch: counter reset");
    launches = 0;
    if (mode == 1) {
        rc = launch_fwdadj(s);
    } else {
        LSS_CUDA_TRY(cudaMemcpyAsync(state.p, d_payoff.p, total_n * sizeof(T), cudaMemcpyDeviceToDevice, s),
                     "batch: initial state");
        rc = launch_forward(s);
    }
    return rc;
}

// Times one run per cap on the warps per instance (32, 64 and 128 threads: groups of at most 1,
// 2 or 4 warps) and keeps the fastest for `mode`; with *chosen > 0 on entry (32, 64, 96 or 128),
// sets that cap without timing.
template <typename T> int batch_typed<T>::autotune(int mode, int *chosen, cudaStream_t s)
{
    const int m = mode == 1 ? 1 : 0;
    if (mode == 1 && !adjoint_ok) return set_error(LSS_ADI_EUNSUPPORTED, "batch: " + adjoint_why);
    if (chosen && *chosen > 0) {
        if (*chosen != 32 && *chosen != 64 && *chosen != 96 && *chosen != 128)
            return set_error(LSS_ADI_EINVAL, "autotune: threads per instance must be 32, 64, 96 or 128");
        bs_mode[m] = *chosen;
        int rc = make_plan(m);
        if (rc) return rc;
    } else {
        const int cand[3] = {32, 64, 128};
        float best = 1e30f;
        int best_bs = bs_mode[m];
        cudaEvent_t e0, e1;
        LSS_CUDA_TRY(cudaEventCreate(&e0), "autotune: event");
        LSS_CUDA_TRY(cudaEventCreate(&e1), "autotune: event");
        for (int c : cand) {
            bs_mode[m] = c;
            int rc = make_plan(m);
            if (rc == LSS_ADI_ENOMEM) { // a plan whose workspace does not fit is skipped
                clear_error();
                continue;
            }
            if (!rc) {
                cudaEventRecord(e0, s);
                rc = enqueue(mode, s);
                cudaEventRecord(e1, s);
            }
            if (rc) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return rc;
            }
            LSS_CUDA_TRY(cudaEventSynchronize(e1), "autotune: run");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                best_bs = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        bs_mode[m] = best_bs;
        int rc = make_plan(m);
        if (rc) return rc;
    }
    if (chosen) *chosen = bs_mode[m];
    return LSS_ADI_OK;
}

// S and v sweeps of the wide path: thread per line (P = 1, bit-identical to the batched
// kernel) or the partitioned solve with the autotuned chunk counts.
template <typename T>
template <int KIND>
void batch_typed<T>::launch_wide_s(cudaStream_t s, const bparams<T> &p, const T *U, const T *Y1, const T *Y2, T *Y)
{
    const bdesc &d = desc[0];
    if (wide_ps <= 1) {
        k_wide_s<T, KIND><<<grid_for(d.ny - 2, 32), 32, 0, s>>>(p, U, Y1, Y2, Y);
    } else {
        const long long n = total_n;
        k_wide_s_chunk<T, KIND><<<grid_for(d.ny - 2, wide_ls), dim3(wide_ls, wide_ps), 0, s>>>(p, U, Y1, Y2, Y, d_spk.p,
                                                                                              d_spk.p + n);
    }
}

template <typename T>
void batch_typed<T>::launch_wide_v(cudaStream_t s, const bparams<T> &p, const T *in, const T *inh, const T *b0, T *out)
{
    const bdesc &d = desc[0];
    if (wide_pv <= 1) {
        if (wide_vtile)
            k_wide_v<T, true><<<grid_for(d.nx - 2, 32), 32, 0, s>>>(p, in, inh, b0, out);
        else
            k_wide_v<T, false><<<grid_for(d.nx - 2, 32), 32, 0, s>>>(p, in, inh, b0, out);
    } else {
        const long long n = total_n;
        if (wide_vtile) {
            const size_t smem = sizeof(vtile<T>) * ((wide_lv * wide_pv) / 32);
            k_wide_v_chunk<T><<<grid_for(d.nx - 2, wide_lv), dim3(wide_lv, wide_pv), smem, s>>>(
                p, in, inh, b0, out, d_spk.p + 2 * n, d_spk.p + 3 * n);
        } else {
            k_wide_v_chunk_plain<T><<<grid_for(d.nx - 2, wide_lv), dim3(wide_lv, wide_pv), 0, s>>>(
                p, in, inh, b0, out, d_spk.p + 2 * n, d_spk.p + 3 * n);
        }
    }
}

template <typename T> int batch_typed<T>::set_wide_chunks(int ps, int pv, cudaStream_t s, int ls, int lv)
{
    const bdesc &d = desc[0];
    const long long n = total_n;
    auto ok = [](int P, int e) { return P >= 1 && P <= MAX_CHUNKS && (P == 1 || e >= 4 * P); };
    if (!ok(ps, d.nx - 2) || !ok(pv, d.ny - 2)) return set_error(LSS_ADI_EINVAL, "wide: chunk count out of range");
    if ((ps > 1 || pv > 1) && !d_spk.p) LSS_CUDA_TRY(d_spk.alloc(4 * n), "wide: allocating chunk products");
    const bparams<T> p = params();
    if (ps > 1)
        k_wide_spikes<T><<<grid_for((d.ny - 2) * ps, 128), 128, 0, s>>>(p.S[SL_LA], p.S[SL_G], d_spk.p, d_spk.p + n, d.ny,
                                                                         d.ny, d.nx - 2, ps);
    if (pv > 1)
        k_wide_spikes<T><<<grid_for((d.nx - 2) * pv, 128), 128, 0, s>>>(p.Vt[VL_LA], p.Vt[VL_G], d_spk.p + 2 * n,
                                                                         d_spk.p + 3 * n, d.nx, d.nx, d.ny - 2, pv);
    LSS_CUDA_TRY(cudaGetLastError(), "wide: chunk products");
    wide_ps = ps;
    wide_pv = pv;
    // the fewest lines per CTA (32, 16 or 8: a warp still reads whole 64-256 B row segments) that
    // give every SM a CTA: with 1-2 k lines, 32 lines per CTA would leave most SMs idle
    auto lines_per_cta = [&](int lines) {
        for (int l : {32, 16})
            if (grid_for(lines, l) >= sms) return l;
        return 8;
    };
    wide_ls = (ls == 8 || ls == 16 || ls == 32) ? ls : lines_per_cta(d.ny - 2);
    wide_lv = (lv == 8 || lv == 16 || lv == 32) ? lv : lines_per_cta(d.nx - 2);
    // the partitioned v sweep works in whole warps (shared-memory tiles moved by all 32 lanes):
    // lines x chunks must be a multiple of 32, which 32 lines per CTA always are
    if (pv > 1 && (wide_lv * pv) % 32 != 0) wide_lv = 32;
    // at most 1024 threads per CTA: 64 chunks take at most 16 lines
    while (ps > 1 && wide_ls * ps > 1024) wide_ls >>= 1;
    while (pv > 1 && wide_lv * pv > 1024) wide_lv >>= 1;
    if (pv > 1) {
        // the limit belongs to the kernel, shared by every solver of the process: set it to what a
        // 1024-thread CTA needs, so that no solver lowers it under another one's launches
        const int smem = static_cast<int>(sizeof(vtile<T>) * 32);
        LSS_CUDA_TRY(cudaFuncSetAttribute(k_wide_v_chunk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                     "wide: v-sweep tile memory");
    }
    if (wide_graph) cudaGraphExecDestroy(wide_graph);
    wide_graph = nullptr;
    return LSS_ADI_OK;
}

// Chunk counts and lines per CTA of the two sweeps, each timed on its own (first S stage,
// first v stage) over P = 1, 2, 4, ..., MAX_CHUNKS (at least 4 rows per chunk) and L = 8, 16,
// 32 (L * P <= 1024).
template <typename T> int batch_typed<T>::autotune_wide(cudaStream_t s)
{
    const bdesc &d = desc[0];
    bparams<T> p = params();
    LSS_CUDA_TRY(cudaMemcpyAsync(p.U, d_payoff.p, total_n * sizeof(T), cudaMemcpyDeviceToDevice, s), "wide: tuning state");
    cudaEvent_t e0, e1;
    LSS_CUDA_TRY(cudaEventCreate(&e0), "wide: tuning events");
    LSS_CUDA_TRY(cudaEventCreate(&e1), "wide: tuning events");
    float best_s = 1e30f, best_v = 1e30f;
    int ps = 1, pv = 1, ls = 32, lv = 32;
    bool vt = true;
    int rc = LSS_ADI_OK;
    auto timed = [&](auto &&launch) {
        launch();
        cudaEventRecord(e0, s);
        for (int r = 0; r < 3; ++r) launch();
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms;
    };
    for (int P = 1; P <= MAX_CHUNKS && rc == LSS_ADI_OK; P *= 2) {
        const bool okS = (P == 1 || d.nx - 2 >= 4 * P), okV = (P == 1 || d.ny - 2 >= 4 * P);
        if (!okS && !okV) break;
        for (int L : {8, 16, 32}) {
            if (P == 1 && L != 32) continue; // thread per line: L unused
            if (L * P > 1024) continue;
            rc = set_wide_chunks(okS ? P : 1, okV ? P : 1, s, L, L);
            if (rc) break;
            if (okS) {
                const float ms = timed([&] { launch_wide_s<1>(s, p, p.U, nullptr, nullptr, p.Y1); });
                if (ms < best_s) { best_s = ms; ps = P; ls = L; }
            }
            if (okV) {
                k_wide_b1<T><<<grid_for(d.nx, 128), 128, 0, s>>>(p, p.U, d_b0.p);
                for (bool tile : {true, false}) {
                    wide_vtile = tile;
                    const float ms = timed([&] { launch_wide_v(s, p, p.U, p.Y1, d_b0.p, p.Y2); });
                    if (ms < best_v) { best_v = ms; pv = P; lv = L; vt = tile; }
                }
            }
            const cudaError_t err = cudaGetLastError();
            if (err != cudaSuccess) {
                rc = set_error(LSS_ADI_ECUDA, std::string("wide: tuning: ") + cudaGetErrorString(err));
                break;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    wide_vtile = vt;
    return set_wide_chunks(ps, pv, s, ls, lv);
}

// One time step U -> V of the wide path (stage outputs in Y1, Y2, Y3).
template <typename T>
void batch_typed<T>::enqueue_wide_step(cudaStream_t s, const bparams<T> &p, const T *U, T *Y1, T *Y2, T *Y3, T *V)
{
    const bdesc &d = desc[0];
    T *b0 = d_b0.p;
    k_wide_b1<T><<<grid_for(d.nx, 128), 128, 0, s>>>(p, U, b0);
    launch_wide_s<1>(s, p, U, nullptr, nullptr, Y1);
    if (d.scheme == LSS_ADI_DOUGLAS_RACHFORD) {
        launch_wide_v(s, p, U, Y1, b0, V);
    } else {
        launch_wide_v(s, p, U, Y1, b0, Y2);
        launch_wide_s<2>(s, p, U, Y1, Y2, Y3);
        if (d.scheme == LSS_ADI_HUNDSDORFER_VERWER)
            launch_wide_v(s, p, Y2, Y3, b0, V);
        else
            launch_wide_v(s, p, U, Y3, b0, V);
    }
    k_wide_b2<T><<<grid_for(d.ny, 128), 128, 0, s>>>(p, V);
}

template <typename T> int batch_typed<T>::enqueue_wide(cudaStream_t s)
{
    const bdesc &d = desc[0];
    bparams<T> p = params();
    T *U = p.U, *V = p.V, *Y1 = p.Y1, *Y2 = p.Y2, *Y3 = p.Y3;
    LSS_CUDA_TRY(cudaMemcpyAsync(U, d_payoff.p, total_n * sizeof(T), cudaMemcpyDeviceToDevice, s), "wide: initial state");
    LSS_CUDA_TRY(cudaMemsetAsync(d_status.p, 0, sizeof(int), s), "wide: clearing the status");
    long long nl = 0;
    const int per_refresh = 3 + (wide_ps > 1 ? 1 : 0);
    for (int step = 0; step < d.steps; ++step) {
        if (tdep) {
            refresh_step(s, step, 1);
            nl += per_refresh;
        }
        enqueue_wide_step(s, p, U, Y1, Y2, Y3, V);
        nl += d.scheme == LSS_ADI_DOUGLAS_RACHFORD ? 4 : 6;
        std::swap(U, V);
    }
    k_wide_finish<T><<<grid_for(total_n, 256), 256, 0, s>>>(p, U);
    LSS_CUDA_TRY(cudaGetLastError(), "wide: launching the time loop");
    launches = nl + 1;
    return LSS_ADI_OK;
}

// Forward + adjoint of the single instance with the wide kernels: forward pass keeping a
// checkpoint every d.ck steps, then per segment (last first) a forward recomputation keeping
// every step's stage values and the adjoint steps in reverse order (as k_batch_fwdadj).
template <typename T> int batch_typed<T>::enqueue_wide_adjoint(cudaStream_t s)
{
    if constexpr (!std::is_same<T, double>::value) {
        (void)s;
        return set_error(LSS_ADI_EUNSUPPORTED, "wide adjoint: FP64 only");
    } else {
        if (count != 1) return set_error(LSS_ADI_EINVAL, "wide adjoint: one instance only");
        if (!adjoint_ok) return set_error(LSS_ADI_EUNSUPPORTED, "wide adjoint: " + adjoint_why);
        bdesc &d = desc[0];
        const int c0 = ck_override > 0 ? std::min(ck_override, d.steps) : d.ck;
        if (c0 != d.ck) {
            d.ck = c0;
            LSS_CUDA_TRY(cudaMemcpy(d_desc.p, &d, sizeof(bdesc), cudaMemcpyHostToDevice), "wide adjoint: descriptor");
        }
        const int nx = d.nx, ny = d.ny, c = d.ck;
        const long long n = total_n;
        const int nseg = (d.steps + c - 1) / c;
        const int threads = 128, grid = grid_for(std::max(nx, ny), threads);
        const long long nthr = static_cast<long long>(grid) * threads;
        // partitioned adjoint solves with the forward's chunk counts
        const int ps = wide_ps, pv = wide_pv, ls = wide_ls, lv = wide_lv;
        const int gS = grid_for(ny - 2, ls), gV = grid_for(nx - 2, lv);
        const long long nacc = std::max({nthr, 1LL * ls * gS * ps, 1LL * lv * gV * pv, static_cast<long long>(nx)});
        if ((ps > 1 || pv > 1) && (aspk_ps != ps || aspk_pv != pv)) {
            if (!d_aspk.p) LSS_CUDA_TRY(d_aspk.alloc(4 * n), "wide adjoint: allocating chunk products");
            const bparams<double> q = params();
            if (ps > 1)
                k_wadj_spikes<double><<<grid_for((ny - 2) * ps, 128), 128, 0, s>>>(q.S[SL_LA], q.S[SL_G], d_aspk.p,
                                                                                   d_aspk.p + n, ny, ny, nx - 2, ps);
            if (pv > 1)
                k_wadj_spikes<double><<<grid_for((nx - 2) * pv, 128), 128, 0, s>>>(q.Vt[VL_LA], q.Vt[VL_G], d_aspk.p + 2 * n,
                                                                                   d_aspk.p + 3 * n, nx, nx, ny - 2, pv);
            LSS_CUDA_TRY(cudaGetLastError(), "wide adjoint: chunk products");
            aspk_ps = ps;
            aspk_pv = pv;
        }
        const double *hzS = d_aspk.p, *hwS = d_aspk.p + n, *hzV = d_aspk.p + 2 * n, *hwV = d_aspk.p + 3 * n;
        const long long need = (nseg + 4LL * (c + 1) + 9) * n + nx + 2LL * ny + 10 * nacc;
        if (!d_wws.p || wws_need != need) {
            LSS_CUDA_TRY(d_wws.alloc(need), "wide adjoint: allocating workspace");
            wws_need = need;
        }
        double *CK = d_wws.p;
        double *SEG = CK + static_cast<long long>(nseg) * n;
        double *W0 = SEG + (c + 1) * 4LL * n, *W1 = W0 + n;
        double *UB = W1 + n, *VB = UB + n, *Y1B = VB + n, *Y2B = Y1B + n, *Y3B = Y2B + n, *FB = Y3B + n, *TMP = FB + n;
        double *LV = TMP + n, *LS = LV + nx, *HS = LS + ny, *ACC = HS + ny;
        auto slot = [&](int m, int a) -> double * { return SEG + (static_cast<long long>(m) * 4 + a) * n; };
        const bparams<double> p = params();
        // stage arrays start at zero (rows 0 and nx-1 of Y2 are never written by the sweeps)
        LSS_CUDA_TRY(cudaMemsetAsync(SEG, 0, (c + 1) * 4LL * n * sizeof(double), s), "wide adjoint: clearing");
        LSS_CUDA_TRY(cudaMemsetAsync(ACC, 0, 10 * nacc * sizeof(double), s), "wide adjoint: clearing");
        LSS_CUDA_TRY(cudaMemsetAsync(d_status.p, 0, sizeof(int), s), "wide adjoint: clearing");
        LSS_CUDA_TRY(cudaMemcpyAsync(CK, d_payoff.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s), "wide adjoint: initial state");
        long long nl = 0;
        const int per_step = d.scheme == LSS_ADI_DOUGLAS_RACHFORD ? 4 : 6;
        const double *cur = CK;
        const int n0_last = (nseg - 1) * c; // the last segment keeps its stage values: no recomputation
        const int per_refresh = 3 + (ps > 1 ? 1 : 0);
        for (int step = 0; step < d.steps; ++step) {
            if (tdep) {
                refresh_step(s, step, 1);
                nl += per_refresh;
            }
            if (step >= n0_last) {
                const int m = step - n0_last;
                enqueue_wide_step(s, p, cur, slot(m, 1), slot(m, 2), slot(m, 3), slot(m + 1, 0));
                nl += per_step;
                cur = slot(m + 1, 0);
                continue;
            }
            double *next = ((step + 1) % c == 0 && step + 1 < d.steps) ? CK + static_cast<long long>((step + 1) / c) * n
                                                                        : ((step & 1) ? W1 : W0);
            enqueue_wide_step(s, p, cur, slot(0, 1), slot(0, 2), slot(0, 3), next);
            nl += per_step;
            cur = next;
        }
        k_wadj_begin<<<grid_for(n, 256), 256, 0, s>>>(p, cur, VB, FB, Y1B, Y3B);
        k_wadj_seed<<<1, 1, 0, s>>>(p, cur, VB);
        nl += 2;
        double *ub = UB, *vb = VB;
        for (int sgi = nseg - 1; sgi >= 0; --sgi) {
            const int n0 = sgi * c;
            const int L = std::min(c, d.steps - n0);
            const double *u0 = CK + static_cast<long long>(sgi) * n;
            for (int m = 0; m < L && sgi < nseg - 1; ++m) {
                const double *um = (m == 0) ? u0 : slot(m, 0);
                if (tdep) {
                    refresh_step(s, n0 + m, 1);
                    nl += per_refresh;
                }
                enqueue_wide_step(s, p, um, slot(m, 1), slot(m, 2), slot(m, 3), slot(m + 1, 0));
                nl += per_step;
            }
            for (int m = L - 1; m >= 0; --m) {
                const double *um = (m == 0) ? u0 : slot(m, 0);
                if (tdep) { // this step's S-line tables and the adjoint's D(t) factors
                    refresh_step(s, n0 + m, 2);
                    nl += per_refresh;
                }
                const double *Y1 = slot(m, 1), *Y2 = slot(m, 2), *Y3 = slot(m, 3), *Vo = slot(m + 1, 0);
                const double tau = d.a_tau0 + d.a_dtau * (n0 + m);
                // v stages: (in, out, output adjoint, adjoint of in, adjoint of inh), first or accumulating
                auto adj_v_stage = [&](bool first, const double *in, const double *out, const double *XB, double *INB,
                                       double *INHB) {
                    if (pv > 1) {
                        if (first)
                            k_wadj_v_chunk<true><<<gV, dim3(lv, pv), 0, s>>>(p, in, out, XB, INB, INHB, TMP, LV, ACC, nacc, hzV, hwV);
                        else
                            k_wadj_v_chunk<false><<<gV, dim3(lv, pv), 0, s>>>(p, in, out, XB, INB, INHB, TMP, LV, ACC, nacc, hzV, hwV);
                    } else {
                        if (first)
                            k_wadj_v<true><<<grid, threads, 0, s>>>(p, in, out, XB, INB, INHB, TMP, LV, ACC, nacc);
                        else
                            k_wadj_v<false><<<grid, threads, 0, s>>>(p, in, out, XB, INB, INHB, TMP, LV, ACC, nacc);
                    }
                };
                auto adj_s_stage = [&](int kind, const double *Yo, const double *XB) {
                    if (ps > 1) {
                        if (kind == 2)
                            k_wadj_s_chunk<2><<<gS, dim3(ls, ps), 0, s>>>(p, um, Y1, Y2, Yo, XB, FB, TMP, LS, HS, ub, Y1B, ACC,
                                                                          nacc, tau, hzS, hwS);
                        else
                            k_wadj_s_chunk<1><<<gS, dim3(ls, ps), 0, s>>>(p, um, Y1, Y2, Yo, XB, FB, TMP, LS, HS, ub, Y1B, ACC,
                                                                          nacc, tau, hzS, hwS);
                    } else {
                        if (kind == 2)
                            k_wadj_s<2><<<grid, threads, 0, s>>>(p, um, Y1, Y2, Yo, XB, FB, TMP, LS, HS, ub, Y1B, ACC, nacc, tau);
                        else
                            k_wadj_s<1><<<grid, threads, 0, s>>>(p, um, Y1, Y2, Yo, XB, FB, TMP, LS, HS, ub, Y1B, ACC, nacc, tau);
                    }
                };
                const int gG = grid_for(n, 256);
                k_wadj_b2<<<grid, threads, 0, s>>>(p, vb, ub);
                if (d.scheme == LSS_ADI_DOUGLAS_RACHFORD) {
                    adj_v_stage(true, um, Vo, vb, ub, Y1B);
                    nl += 2;
                } else {
                    if (d.scheme == LSS_ADI_HUNDSDORFER_VERWER)
                        adj_v_stage(true, Y2, Vo, vb, Y2B, Y3B);
                    else
                        adj_v_stage(true, um, Vo, vb, ub, Y3B);
                    adj_s_stage(2, Y3, Y3B);
                    k_wadj_gather2d<2><<<gG, 256, 0, s>>>(p, um, FB, LS, HS, LV, ub, Y2B, ACC, nacc, tau);
                    adj_v_stage(false, um, Y2, Y2B, ub, Y1B);
                    nl += 5;
                }
                adj_s_stage(1, Y1, Y1B);
                k_wadj_gather2d<1><<<gG, 256, 0, s>>>(p, um, FB, LS, HS, LV, ub, Y2B, ACC, nacc, tau);
                nl += 2;
                std::swap(ub, vb);
            }
        }
        k_wadj_reduce<<<1, 256, 0, s>>>(p, ACC, nacc);
        LSS_CUDA_TRY(cudaMemcpyAsync(p.V, vb, n * sizeof(double), cudaMemcpyDeviceToDevice, s), "wide adjoint: payoff gradient");
        LSS_CUDA_TRY(cudaGetLastError(), "wide adjoint: launching");
        launches = nl + 1;
        return LSS_ADI_OK;
    }
}

template <typename T> int batch_typed<T>::run_wide(cudaStream_t s, bool use_graph)
{
    if (count != 1) return set_error(LSS_ADI_EINVAL, "wide path: one instance only");
    if (!use_graph) return enqueue_wide(s);
    if (!wide_graph) {
        cudaStream_t cs;
        LSS_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "wide: capture stream");
        LSS_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "wide: begin capture");
        const int rc = enqueue_wide(cs);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (rc) return rc;
        LSS_CUDA_TRY(e, "wide: end capture");
        e = cudaGraphInstantiate(&wide_graph, g, 0);
        cudaGraphDestroy(g);
        LSS_CUDA_TRY(e, "wide: instantiate graph");
    }
    LSS_CUDA_TRY(cudaGraphLaunch(wide_graph, s), "wide: graph launch");
    return LSS_ADI_OK;
}

template <typename T> int batch_typed<T>::run(int mode, cudaStream_t s, bool use_graph)
{
    { // plans (allocations, uploads) happen here, never inside a stream capture
        int rc = mode == 1 ? prepare_adjoint(s) : make_plan(0);
        if (rc) return rc;
    }
    if (!use_graph) return enqueue(mode, s);
    if (!graph || graph_mode != mode) {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        cudaStream_t cs;
        LSS_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "batch: capture stream");
        LSS_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "batch: begin capture");
        int rc = enqueue(mode, cs);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (rc) return rc;
        LSS_CUDA_TRY(e, "batch: end capture");
        e = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        LSS_CUDA_TRY(e, "batch: instantiate graph");
        graph_mode = mode;
    }
    LSS_CUDA_TRY(cudaGraphLaunch(graph, s), "batch: graph launch");
    return LSS_ADI_OK;
}

template <typename T> struct wide_solver : wide_solver_base {
    batch_typed<T> b;
    std::vector<T> x, y, pay0;

    int init(const lss_adi_problem &p)
    {
        instance_tables<T> tt;
        build_tables_for<T>(p, tt);
        x = tt.x;
        y = tt.y;
        pay0 = tt.payoff;
        int rc = b.create(&p, 1);
        if (rc) return rc;
        if (p.options & LSS_ADI_OPT_LINE_PER_THREAD) return LSS_ADI_OK;
        LSS_CUDA_TRY(cudaMemcpy(b.d_payoff.p, pay0.data(), pay0.size() * sizeof(T), cudaMemcpyHostToDevice),
                     "wide: initial state");
        rc = b.autotune_wide(nullptr);
        if (rc) return rc;
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "wide: tuning");
        return LSS_ADI_OK;
    }
    int forward(const void *payoff, void *out_surface, double *out_value, int flags, void *stream, bool use_graph) override
    {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const bool dev = (flags & LSS_ADI_DEVICE_POINTERS) != 0;
        const size_t n = static_cast<size_t>(b.total_n);
        const void *src = payoff ? payoff : static_cast<const void *>(pay0.data());
        LSS_CUDA_TRY(cudaMemcpyAsync(b.d_payoff.p, src, n * sizeof(T),
                                     (payoff && dev) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s),
                     "wide: copying the terminal condition");
        int rc = b.run_wide(s, use_graph);
        if (rc) return rc;
        if (out_value)
            LSS_CUDA_TRY(cudaMemcpyAsync(out_value, b.d_values.p, sizeof(double), cudaMemcpyDeviceToHost, s), "wide: value");
        if (out_surface) {
            const T *fin = b.state.p + ((b.desc[0].steps & 1) ? b.total_n : 0);
            LSS_CUDA_TRY(cudaMemcpyAsync(out_surface, fin, n * sizeof(T), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s),
                         "wide: surface");
        }
        if (!dev || out_value) LSS_CUDA_TRY(cudaStreamSynchronize(s), "wide: time loop");
        return LSS_ADI_OK;
    }
    int grid(void *gx, void *gy) const override
    {
        std::copy(x.begin(), x.end(), static_cast<T *>(gx));
        std::copy(y.begin(), y.end(), static_cast<T *>(gy));
        return LSS_ADI_OK;
    }
    int chunks(int s_chunks, int v_chunks, int *out_s, int *out_v, void *stream) override
    {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (s_chunks < 0 || v_chunks < 0) return set_error(LSS_ADI_EINVAL, "lss_adi_line_chunks: negative chunk count");
        int rc = LSS_ADI_OK;
        if (s_chunks == 0 || v_chunks == 0) {
            LSS_CUDA_TRY(cudaMemcpyAsync(b.d_payoff.p, pay0.data(), pay0.size() * sizeof(T), cudaMemcpyHostToDevice, s),
                         "wide: initial state");
            rc = b.autotune_wide(s);
            if (rc) return rc;
        }
        if (s_chunks || v_chunks) { // a direction left at 0 keeps its tuned chunks and lines per CTA
            rc = b.set_wide_chunks(s_chunks ? s_chunks : b.wide_ps, v_chunks ? v_chunks : b.wide_pv, s,
                                   s_chunks ? 0 : b.wide_ls, v_chunks ? 0 : b.wide_lv);
            if (rc) return rc;
        }
        LSS_CUDA_TRY(cudaStreamSynchronize(s), "lss_adi_line_chunks");
        if (out_s) *out_s = b.wide_ps;
        if (out_v) *out_v = b.wide_pv;
        return LSS_ADI_OK;
    }
    void current_chunks(int &s_chunks, int &v_chunks, int &s_lines, int &v_lines) const override
    {
        s_chunks = b.wide_ps;
        v_chunks = b.wide_pv;
        s_lines = b.wide_ls;
        v_lines = b.wide_lv;
    }
};

int make_wide_solver(const lss_adi_problem &p, std::unique_ptr<wide_solver_base> &out)
{
    try {
        if (p.precision == LSS_ADI_FP64) {
            std::unique_ptr<wide_solver<double>> w(new wide_solver<double>());
            int rc = w->init(p);
            if (rc) return rc;
            out = std::move(w);
        } else {
            std::unique_ptr<wide_solver<float>> w(new wide_solver<float>());
            int rc = w->init(p);
            if (rc) return rc;
            out = std::move(w);
        }
    } catch (const std::bad_alloc &) {
        return set_error(LSS_ADI_ENOMEM, "wide: host allocation failed");
    }
    return LSS_ADI_OK;
}

// lss_adi_adjoint: one parametric FP64 Heston instance through the batched forward+adjoint kernel.
struct adjoint_impl {
    batch_typed<double> b;
    bool wide = false; // large instance: the wide kernels instead of one CTA
};

adjoint_solver::adjoint_solver() = default;
adjoint_solver::~adjoint_solver() = default;

int adjoint_solver::init(const lss_adi_problem &p)
{
    if (p.scheme == LSS_ADI_EXPLICIT_EULER)
        return set_error(LSS_ADI_EUNSUPPORTED, "lss_adi_adjoint: no adjoint for the explicit Euler scheme");
    impl.reset(new (std::nothrow) adjoint_impl());
    if (!impl) return set_error(LSS_ADI_ENOMEM, "host allocation failed");
    lss_adi_problem q = p;
    q.arith = LSS_ADI_ARITH_FAST;
    int rc = impl->b.create(&q, 1);
    if (rc) return rc;
    // one CTA carries an instance of up to 256 x 160 points well; larger ones run wide, and so
    // do time-dependent coefficients (SABR with r != 0), whose S-line tables the host-sequenced
    // wide kernels rebuild before every step
    impl->wide = p.nx > 256 || static_cast<long long>(p.nx) * p.ny > 40960 || (p.options & LSS_ADI_OPT_WIDE_ADJOINT) ||
                 time_dependent(p);
    if (impl->wide && !(p.options & LSS_ADI_OPT_LINE_PER_THREAD)) {
        rc = impl->b.autotune_wide(nullptr);
        if (rc) return rc;
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "lss_adi_adjoint: tuning");
    }
    return LSS_ADI_OK;
}

int adjoint_solver::set_chunks(int s_chunks, int v_chunks, int s_lines, int v_lines, void *stream)
{
    if (!impl || !impl->wide) return LSS_ADI_OK;
    return impl->b.set_wide_chunks(s_chunks, v_chunks, static_cast<cudaStream_t>(stream), s_lines, v_lines);
}

int adjoint_solver::run(const void *payoff, double *out_value, double *dv_dparams, void *dv_dpayoff, int checkpoint_every,
                        int flags, void *stream)
{
    batch_typed<double> &b = impl->b;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool dev = (flags & LSS_ADI_DEVICE_POINTERS) != 0;
    const size_t n = static_cast<size_t>(b.total_n);
    if (payoff)
        LSS_CUDA_TRY(cudaMemcpyAsync(b.d_payoff.p, payoff, n * sizeof(double),
                                     dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s),
                     "lss_adi_adjoint: copying the terminal condition");
    b.ck_override = checkpoint_every;
    int rc = impl->wide ? b.enqueue_wide_adjoint(s) : b.run(1, s, false);
    if (rc) return rc;
    if (out_value)
        LSS_CUDA_TRY(cudaMemcpyAsync(out_value, b.d_values.p, sizeof(double), cudaMemcpyDeviceToHost, s), "lss_adi_adjoint: value");
    if (dv_dparams)
        LSS_CUDA_TRY(cudaMemcpyAsync(dv_dparams, b.d_grads.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, s),
                     "lss_adi_adjoint: gradients");
    if (dv_dpayoff)
        LSS_CUDA_TRY(cudaMemcpyAsync(dv_dpayoff, b.state.p + b.total_n, n * sizeof(double),
                                     dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s),
                     "lss_adi_adjoint: payoff gradient");
    LSS_CUDA_TRY(cudaStreamSynchronize(s), "lss_adi_adjoint: run");
    return LSS_ADI_OK;
}

template <typename T> static int set_workspace_t(batch_typed<T> &bt, double max_bytes, int checkpoint_every)
{
    bt.ws_cap = max_bytes;
    bt.ck_override = checkpoint_every;
    if (bt.graph && bt.graph_mode == 1) { // a captured launch holds the old workspace and plan
        cudaGraphExecDestroy(bt.graph);
        bt.graph = nullptr;
        bt.graph_mode = -1;
    }
    return LSS_ADI_OK;
}

template <typename T> static int payoff_grad_t(batch_typed<T> &bt, int index, void *out)
{
    if (index < 0 || index >= bt.count) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_payoff_gradient: index out of range");
    if (!std::is_same<T, double>::value) return set_error(LSS_ADI_EUNSUPPORTED, "lss_adi_batch_payoff_gradient: FP64 only");
    LSS_CUDA_TRY(cudaDeviceSynchronize(), "batch: synchronising");
    const bdesc &d = bt.desc[index];
    LSS_CUDA_TRY(cudaMemcpy(out, bt.state.p + bt.total_n + d.o2, static_cast<size_t>(d.nx) * d.ny * sizeof(T),
                            cudaMemcpyDeviceToHost),
                 "batch: payoff gradient");
    return LSS_ADI_OK;
}

} // namespace lss_gb300

using namespace lss_gb300;

struct lss_adi_batch {
    int precision = LSS_ADI_FP64;
    std::unique_ptr<batch_typed<double>> b64;
    std::unique_ptr<batch_typed<float>> b32;
    cudaStream_t last_stream = nullptr;
};

template <typename T>
static int run_host_t(batch_typed<T> &bt, int mode, const void *payoffs, double *values, double *grads, cudaStream_t s)
{
    if (payoffs)
        LSS_CUDA_TRY(cudaMemcpyAsync(bt.d_payoff.p, payoffs, bt.total_n * sizeof(T), cudaMemcpyHostToDevice, s),
                     "batch: uploading payoffs");
    int rc = bt.run(mode, s, true);
    if (rc) return rc;
    if (values)
        LSS_CUDA_TRY(cudaMemcpyAsync(values, bt.d_values.p, bt.count * sizeof(double), cudaMemcpyDeviceToHost, s),
                     "batch: reading values");
    if (grads && mode == 1)
        LSS_CUDA_TRY(cudaMemcpyAsync(grads, bt.d_grads.p, 5 * bt.count * sizeof(double), cudaMemcpyDeviceToHost, s),
                     "batch: reading gradients");
    LSS_CUDA_TRY(cudaStreamSynchronize(s), "batch: run");
    return LSS_ADI_OK;
}

template <typename T> static int results_t(batch_typed<T> &bt, double *values, double *grads, int *status)
{
    LSS_CUDA_TRY(cudaDeviceSynchronize(), "batch: synchronising");
    if (values) LSS_CUDA_TRY(cudaMemcpy(values, bt.d_values.p, bt.count * sizeof(double), cudaMemcpyDeviceToHost), "batch: values");
    if (status) LSS_CUDA_TRY(cudaMemcpy(status, bt.d_status.p, bt.count * sizeof(int), cudaMemcpyDeviceToHost), "batch: status");
    if (grads) LSS_CUDA_TRY(cudaMemcpy(grads, bt.d_grads.p, 5 * bt.count * sizeof(double), cudaMemcpyDeviceToHost), "batch: grads");
    return LSS_ADI_OK;
}

template <typename T> static int surface_t(batch_typed<T> &bt, int index, void *out)
{
    if (index < 0 || index >= bt.count) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_surface: index out of range");
    LSS_CUDA_TRY(cudaDeviceSynchronize(), "batch: synchronising");
    int fin = 0;
    LSS_CUDA_TRY(cudaMemcpy(&fin, bt.d_final.p + index, sizeof(int), cudaMemcpyDeviceToHost), "batch: flag");
    const bdesc &d = bt.desc[index];
    const T *src = bt.state.p + (fin ? bt.total_n : 0) + d.o2;
    LSS_CUDA_TRY(cudaMemcpy(out, src, static_cast<size_t>(d.nx) * d.ny * sizeof(T), cudaMemcpyDeviceToHost), "batch: surface");
    return LSS_ADI_OK;
}

extern "C" {

int lss_adi_batch_create(const lss_adi_problem *problems, int count, lss_adi_batch **b)
{
    clear_error();
    if (!b) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_create: null output");
    *b = nullptr;
    if (!problems || count <= 0) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_create: empty batch");
    const int prec = problems[0].precision;
    for (int k = 0; k < count; ++k) {
        std::string why;
        int rc = validate_problem(problems[k], why);
        if (rc) return set_error(rc, "lss_adi_batch_create: instance " + std::to_string(k) + ": " + why);
        if (problems[k].precision != prec) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_create: mixed precisions");
        if (problems[k].scheme == LSS_ADI_EXPLICIT_EULER)
            return set_error(LSS_ADI_EUNSUPPORTED, "lss_adi_batch_create: instance " + std::to_string(k) +
                                                       ": the explicit Euler scheme runs on lss_adi_create");
        if (time_dependent(problems[k]))
            return set_error(LSS_ADI_EUNSUPPORTED, "lss_adi_batch_create: instance " + std::to_string(k) +
                                                       ": SABR with r != 0 has time-dependent coefficients (use lss_adi_create)");
    }
    std::unique_ptr<lss_adi_batch> h(new (std::nothrow) lss_adi_batch());
    if (!h) return set_error(LSS_ADI_ENOMEM, "host allocation failed");
    h->precision = prec;
    int rc;
    try {
        if (prec == LSS_ADI_FP64) {
            h->b64.reset(new batch_typed<double>());
            rc = h->b64->create(problems, count);
        } else {
            h->b32.reset(new batch_typed<float>());
            rc = h->b32->create(problems, count);
        }
    } catch (const std::bad_alloc &) {
        return set_error(LSS_ADI_ENOMEM, "lss_adi_batch_create: host allocation failed");
    }
    if (rc) return rc;
    *b = h.release();
    return LSS_ADI_OK;
}

static int batch_run(lss_adi_batch *b, int mode, void *stream, bool graph)
{
    clear_error();
    if (!b) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_run: null batch");
    if (mode != 0 && mode != 1) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_run: mode must be 0 or 1");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    b->last_stream = s;
    return b->b64 ? b->b64->run(mode, s, graph) : b->b32->run(mode, s, graph);
}

int lss_adi_batch_run(lss_adi_batch *b, int mode, void *stream) { return batch_run(b, mode, stream, false); }
int lss_adi_batch_graph_launch(lss_adi_batch *b, int mode, void *stream) { return batch_run(b, mode, stream, true); }


int lss_adi_batch_run_host(lss_adi_batch *b, int mode, const void *payoffs, double *values, double *grads, void *stream)
{
    clear_error();
    if (!b) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_run_host: null batch");
    if (mode != 0 && mode != 1) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_run_host: mode must be 0 or 1");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    b->last_stream = s;
    return b->b64 ? run_host_t(*b->b64, mode, payoffs, values, grads, s)
                  : run_host_t(*b->b32, mode, payoffs, values, grads, s);
}


int lss_adi_batch_results(lss_adi_batch *b, double *values, double *grads, int *status)
{
    clear_error();
    if (!b) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_results: null batch");
    return b->b64 ? results_t(*b->b64, values, grads, status) : results_t(*b->b32, values, grads, status);
}


int lss_adi_batch_surface(lss_adi_batch *b, int index, void *out_surface)
{
    clear_error();
    if (!b || !out_surface) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_surface: null argument");
    return b->b64 ? surface_t(*b->b64, index, out_surface) : surface_t(*b->b32, index, out_surface);
}

int lss_adi_batch_payoff_gradient(lss_adi_batch *b, int index, void *out)
{
    clear_error();
    if (!b || !out) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_payoff_gradient: null argument");
    return b->b64 ? payoff_grad_t(*b->b64, index, out) : payoff_grad_t(*b->b32, index, out);
}

int lss_adi_batch_autotune(lss_adi_batch *b, int mode, int *threads_per_instance, void *stream)
{
    clear_error();
    if (!b) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_autotune: null batch");
    if (mode != 0 && mode != 1) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_autotune: mode must be 0 or 1");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return b->b64 ? b->b64->autotune(mode, threads_per_instance, s) : b->b32->autotune(mode, threads_per_instance, s);
}

int lss_adi_batch_launch_count(const lss_adi_batch *b)
{
    if (!b) return 0;
    return static_cast<int>(b->b64 ? b->b64->launches : b->b32->launches);
}

int lss_adi_batch_checkpoints(const lss_adi_batch *b, int *intervals)
{
    if (!b || !intervals) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_checkpoints: null argument");
    const int count = b->b64 ? b->b64->count : b->b32->count;
    for (int k = 0; k < count; ++k) intervals[k] = b->b64 ? b->b64->desc[k].ck : b->b32->desc[k].ck;
    return LSS_ADI_OK;
}

int lss_adi_batch_set_workspace(lss_adi_batch *b, double max_bytes, int checkpoint_every)
{
    clear_error();
    if (!b) return set_error(LSS_ADI_EINVAL, "lss_adi_batch_set_workspace: null batch");
    if (!(max_bytes >= 0.0) || checkpoint_every < 0)
        return set_error(LSS_ADI_EINVAL, "lss_adi_batch_set_workspace: negative cap or interval");
    return b->b64 ? set_workspace_t(*b->b64, max_bytes, checkpoint_every)
                  : set_workspace_t(*b->b32, max_bytes, checkpoint_every);
}

double lss_adi_batch_workspace_bytes(const lss_adi_batch *b)
{
    if (!b) return 0.0;
    return b->b64 ? static_cast<double>(b->b64->d_ws.n) * sizeof(double) : 0.0;
}

void lss_adi_batch_destroy(lss_adi_batch *b) { delete b; }

} // extern "C"
