// adi_plain.cu -- one instance per launch sequence: one kernel per sweep.
//
// Time step (implicit_heston_time_loop::run, lss_2d_general_heston_equation_implicit_kernel.hpp:150-207):
//   boundary#1 (v = v_lo column explicit, v = v_hi column Dirichlet)     k_boundary1
//   splitting scheme: S-line sweeps (thread per line j, coalesced along j)   k_s_sweep
//                     v-line sweeps (thread per line i)                      k_v_sweep
//                     HV full-grid stage                                     k_hv_stage3
//   boundary#2 (row S_lo Dirichlet, row S_hi extrapolated Neumann)          k_boundary2
//   prev <- next                                                             pointer swap
// State layout: row-major V[i*ny + j] (S index i, v index j), the reference's
// container_2d<by_enum::Row>.
#include "adi_plain.hpp"

#include <algorithm>
#include <vector>

namespace lss_gb300 {

// ------------------------------------------------------------------------------------------
// boundary#1: explicit_heston_boundary_scheme::rhs (explicit_boundary.hpp:39-84) + v_hi column
// ------------------------------------------------------------------------------------------
// Results go to bcol0[i * stride], bcolN[i * stride]: the boundary columns of the v lines
// (stride 1) or, for the explicit Euler step, columns 0 and ny-1 of the next state (stride ny).
template <typename T, bool X>
__global__ void k_boundary1(dev_instance<T> d, const T *__restrict__ U, T *__restrict__ bcol0, T *__restrict__ bcolN,
                            int stride)
{
    using R = ar<X>;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = d.nx, ny = d.ny, N = nx - 1;
    if (i >= nx) return;
    const T one = T(1), two = T(2), three = T(3), four = T(4);
    const long long w = static_cast<long long>(i) * stride;
    if (i == 0) {
        bcol0[0] = d.s_lo[0];
    } else if (i == N) {
        const T D = d.D0[N], E = d.E0[N], F = d.F0[N];
        const T dlt = R::mul(R::mul(two, d.h1), d.s_hi_neu[0]);
        const T t1 = R::mul(R::add(R::sub(one, R::mul(R::mul(three, d.ni), E)), R::mul(d.rho, F)), U[N * ny]);
        const T t2 = R::mul(R::mul(R::mul(four, d.ni), E), U[N * ny + 1]);
        const T t3 = R::mul(R::mul(d.ni, E), U[N * ny + 2]);
        const T t4 = R::mul(R::mul(d.delta, dlt), D);
        bcol0[w] = R::sub(R::sub(R::add(t1, t2), t3), t4);
    } else {
        const T D = d.D0[i], E = d.E0[i], F = d.F0[i];
        const T t1 = R::mul(R::mul(-d.delta, D), U[(i - 1) * ny]);
        const T t2 = R::mul(R::add(R::sub(one, R::mul(R::mul(three, d.ni), E)), R::mul(d.rho, F)), U[i * ny]);
        const T t3 = R::mul(R::mul(d.delta, D), U[(i + 1) * ny]);
        const T t4 = R::mul(R::mul(d.ni, E), U[i * ny + 2]);
        const T t5 = R::mul(R::mul(R::mul(four, d.ni), E), U[i * ny + 1]);
        bcol0[w] = R::add(R::sub(R::add(R::add(t1, t2), t3), t4), t5);
    }
    bcolN[w] = d.v_hi[i];
}

// ------------------------------------------------------------------------------------------
// One forward step of double_sweep_solver (lss_double_sweep_solver.hpp:114-155 with the
// Dirichlet start L = 0, K = lo of lss_double_sweep_boundary.hpp:90-190):
//   tmp = b + a*L;  L' = (-1*c)/tmp;  K' = (f - a*K)/tmp
// and back substitution x_t = L_t*x_{t+1} + K_t from x_{n-1} = hi.
// ------------------------------------------------------------------------------------------
template <bool X, typename T> __device__ __forceinline__ void ds_forward(T a, T b, T c, T f, T &L, T &K)
{
    using R = ar<X>;
    const T tmp = R::add(b, R::mul(a, L));
    L = R::div(R::mul(T(-1), c), tmp);
    K = R::div(R::sub(f, R::mul(a, K)), tmp);
}

// ------------------------------------------------------------------------------------------
// S-line sweep: line j = 1..ny-2 solves rows 1..nx-2 of column j with Dirichlet ends
// prev(0, jmap[j]) and prev(nx-1, jmap[j]) (get_intermed_horizontal, implicit_kernel.hpp:86-101);
// matrix split_0 (lss_heat_douglas_rachford_method.hpp:159-169); Thomas LU in the
// reference order (lss_thomas_lu_solver.hpp:161-190), or the double sweep when d.ds is set.
// Y receives the whole column incl. ends.
// ------------------------------------------------------------------------------------------
template <typename T, bool X, int STAGE>
__global__ void k_s_sweep(dev_instance<T> d, const T *__restrict__ Ub, const T *__restrict__ A,
                          const T *__restrict__ B, const T *__restrict__ Cc, T *__restrict__ Y, T *__restrict__ G)
{
    using R = ar<X>;
    const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = d.nx, ny = d.ny;
    if (j > ny - 2) return;
    const int jj = d.jmap[j];
    const T lo = Ub[jj], hi = Ub[(nx - 1) * ny + jj];
    const T one = T(1);
    const int e = nx - 2;
    if (d.ds) {
        // double_sweep_solver: L/K recurrences, L in G and K in Y
        T L = T(0), K = lo;
        for (int t = 1; t <= e; ++t) {
            const int o = t * ny + j;
            const T a = R::mul(-d.theta, d.M[o]);
            const T tz = R::mul(d.theta, d.Z[o]);
            const T b = R::add(one, tz);
            const T tp = R::mul(d.theta, d.P[o]);
            const T c = -tp;
            const T f = s_rhs<T, X, STAGE>(d, t, j, A, B, Cc, a, tz, tp);
            ds_forward<X>(a, b, c, f, L, K);
            G[o] = L;
            Y[o] = K;
        }
        T x = hi;
        for (int t = e; t >= 1; --t) {
            const int o = t * ny + j;
            x = R::add(R::mul(G[o], x), Y[o]);
            Y[o] = x;
        }
        Y[j] = lo;
        Y[(nx - 1) * ny + j] = hi;
        return;
    }
    T gam = T(0), y = T(0);
    for (int t = 1; t <= e; ++t) {
        const int o = t * ny + j;
        const T a = R::mul(-d.theta, d.M[o]);
        const T tz = R::mul(d.theta, d.Z[o]);
        const T b = R::add(one, tz);
        const T tp = R::mul(d.theta, d.P[o]);
        const T c = -tp;
        const T f = s_rhs<T, X, STAGE>(d, t, j, A, B, Cc, a, tz, tp);
        if (t == 1) {
            const T beta = b;
            gam = R::div(c, beta);
            y = R::div(R::sub(f, R::mul(a, lo)), beta);
        } else if (t < e) {
            const T beta = R::sub(b, R::mul(a, gam));
            y = R::div(R::sub(f, R::mul(a, y)), beta);
            gam = R::div(c, beta);
        } else {
            const T beta = R::sub(b, R::mul(a, gam));
            y = R::div(R::sub(R::sub(f, R::mul(c, hi)), R::mul(a, y)), beta);
        }
        G[o] = gam;
        Y[o] = y;
    }
    T x = y;
    for (int t = e - 1; t >= 1; --t) {
        const int o = t * ny + j;
        x = R::sub(Y[o], R::mul(G[o], x));
        Y[o] = x;
    }
    Y[j] = lo;
    Y[(nx - 1) * ny + j] = hi;
}

// ------------------------------------------------------------------------------------------
// v-line sweep: line i = 1..nx-2 solves columns 1..ny-2 of row i with Dirichlet ends
// bcol0[imap[i]], bcolN[imap[i]] (get_vertical, implicit_kernel.hpp:69-84); matrix split_1
// (:171-181); right-hand side rhs / rhs_intermed_2 / rhs_final (:106-126).
// ------------------------------------------------------------------------------------------
template <typename T, bool X>
__global__ void k_v_sweep(dev_instance<T> d, const T *__restrict__ in, const T *__restrict__ inh,
                          const T *__restrict__ bcol0, const T *__restrict__ bcolN, T *__restrict__ out,
                          T *__restrict__ G)
{
    using R = ar<X>;
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = d.nx, ny = d.ny;
    if (i > nx - 2) return;
    const int ii = d.imap[i];
    const T lo = bcol0[ii], hi = bcolN[ii];
    const T one = T(1);
    const int e = ny - 2;
    const int row = i * ny;
    if (d.ds) {
        T L = T(0), K = lo;
        for (int t = 1; t <= e; ++t) {
            const int o = row + t;
            const T a = R::mul(-d.theta, d.Mt[o]);
            const T tw = R::mul(d.theta, d.W[o]);
            const T b = R::add(one, tw);
            const T tp = R::mul(d.theta, d.Pt[o]);
            const T c = -tp;
            const T f = R::add(R::sub(R::add(R::mul(a, in[o - 1]), R::mul(tw, in[o])), R::mul(tp, in[o + 1])), inh[o]);
            ds_forward<X>(a, b, c, f, L, K);
            G[o] = L;
            out[o] = K;
        }
        T x = hi;
        for (int t = e; t >= 1; --t) {
            const int o = row + t;
            x = R::add(R::mul(G[o], x), out[o]);
            out[o] = x;
        }
        out[row] = lo;
        out[row + ny - 1] = hi;
        return;
    }
    T gam = T(0), y = T(0);
    for (int t = 1; t <= e; ++t) {
        const int o = row + t;
        const T a = R::mul(-d.theta, d.Mt[o]);
        const T tw = R::mul(d.theta, d.W[o]);
        const T b = R::add(one, tw);
        const T tp = R::mul(d.theta, d.Pt[o]);
        const T c = -tp;
        const T f = R::add(R::sub(R::add(R::mul(a, in[o - 1]), R::mul(tw, in[o])), R::mul(tp, in[o + 1])), inh[o]);
        if (t == 1) {
            const T beta = b;
            gam = R::div(c, beta);
            y = R::div(R::sub(f, R::mul(a, lo)), beta);
        } else if (t < e) {
            const T beta = R::sub(b, R::mul(a, gam));
            y = R::div(R::sub(f, R::mul(a, y)), beta);
            gam = R::div(c, beta);
        } else {
            const T beta = R::sub(b, R::mul(a, gam));
            y = R::div(R::sub(R::sub(f, R::mul(c, hi)), R::mul(a, y)), beta);
        }
        G[o] = gam;
        out[o] = y;
    }
    T x = y;
    for (int t = e - 1; t >= 1; --t) {
        const int o = row + t;
        x = R::sub(out[o], R::mul(G[o], x));
        out[o] = x;
    }
    out[row] = lo;
    out[row + ny - 1] = hi;
}

// ------------------------------------------------------------------------------------------
// Explicit Euler interior (explicit_heston_scheme::rhs, solver_method/
// lss_heston_euler_solver_method.hpp:24-52, in its evaluation order): the 9-point operator on
// `U` with the Euler mixed weight gamma * C (explicit_coefficients/lss_heston_euler_coefficients.hpp:53).
// ------------------------------------------------------------------------------------------
template <typename T, bool X>
__global__ void k_euler(dev_instance<T> d, const T *__restrict__ U, T *__restrict__ V)
{
    using R = ar<X>;
    const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int i = 1 + blockIdx.y;
    const int ny = d.ny;
    if (j > ny - 2) return;
    const long long o = static_cast<long long>(i) * ny + j;
    const T one = T(1);
    const T C = R::mul(d.gamma, d.C[o]);
    T v = R::mul(C, U[o - ny - 1]);
    v = R::add(v, R::mul(d.M[o], U[o - ny]));
    v = R::sub(v, R::mul(C, U[o - ny + 1]));
    v = R::add(v, R::mul(d.Mt[o], U[o - 1]));
    v = R::add(v, R::mul(R::sub(R::sub(one, d.Z[o]), d.W[o]), U[o]));
    v = R::add(v, R::mul(d.Pt[o], U[o + 1]));
    v = R::sub(v, R::mul(C, U[o + ny - 1]));
    v = R::add(v, R::mul(d.P[o], U[o + ny]));
    v = R::add(v, R::mul(C, U[o + ny + 1]));
    V[o] = v;
}

// ------------------------------------------------------------------------------------------
// HV full-grid stage rhs_intermed_3 (lss_heat_hundsdorfer_verwer_method.hpp:146-171).
// ------------------------------------------------------------------------------------------
template <typename T, bool X>
__global__ void k_hv_stage3(dev_instance<T> d, const T *__restrict__ U, const T *__restrict__ Y1,
                            const T *__restrict__ Y2, T *__restrict__ Y3)
{
    using R = ar<X>;
    const int nx = d.nx, ny = d.ny;
    const int q = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int r = 1 + blockIdx.y;
    if (q > ny - 2 || r > nx - 2) return;
    const int o = r * ny + q;
    const T one = T(1);
    const T th = d.theta;
    const T M = d.M[o], Z = d.Z[o], P = d.P[o], W = d.W[o];
    const T t1 = R::mul(R::mul(-th, M), Y1[o - ny]);
    const T t2 = R::mul(R::add(one, R::mul(th, Z)), Y1[o]);
    const T t3 = R::mul(R::mul(th, P), Y1[o + ny]);
    const T t4 = R::mul(R::mul(th, M), U[o - ny]);
    const T t5 = R::mul(R::mul(th, Z), U[o]);
    const T t6 = R::mul(R::mul(th, P), U[o + ny]);
    const T d1 = R::sub(Y2[o + ny + 1], U[o + ny + 1]);
    const T d2 = R::sub(Y2[o + ny - 1], U[o + ny - 1]);
    const T d3 = R::sub(Y2[o - ny + 1], U[o - ny + 1]);
    const T d4 = R::sub(Y2[o - ny - 1], U[o - ny - 1]);
    const T t7 = R::mul(R::mul(R::mul(d.zeta, d.gamma), d.C[o]), R::add(R::sub(R::sub(d1, d2), d3), d4));
    const T e1 = R::mul(M, R::sub(Y2[o - ny], U[o - ny]));
    const T e2 = R::mul(R::add(W, Z), R::sub(Y2[o], U[o]));
    const T e3 = R::mul(P, R::sub(Y2[o + ny], U[o + ny]));
    const T e4 = R::mul(d.Mt[o], R::sub(Y2[o - 1], U[o - 1]));
    const T e5 = R::mul(d.Pt[o], R::sub(Y2[o + 1], U[o + 1]));
    const T t8 = R::mul(d.zeta, R::add(R::add(R::add(R::sub(e1, e2), e3), e4), e5));
    Y3[o] = R::add(R::add(R::add(R::sub(R::add(R::sub(R::add(t1, t2), t3), t4), t5), t6), t7), t8);
}

// ------------------------------------------------------------------------------------------
// boundary#2 (explicit_boundary.hpp:202-238): row 0 Dirichlet, row nx-1 from the
// one-sided Neumann extrapolation with the index_of-remapped column.
// ------------------------------------------------------------------------------------------
template <typename T, bool X> __global__ void k_boundary2(dev_instance<T> d, T *__restrict__ V)
{
    using R = ar<X>;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = d.nx, ny = d.ny;
    if (j >= ny) return;
    const T two = T(2), three = T(3), four = T(4);
    V[j] = d.s_lo[j];
    const int jj = d.jmap[j];
    const int lri = nx - 1;
    V[lri * ny + j] = R::div(R::sub(R::sub(R::mul(four, V[(lri - 1) * ny + jj]), V[(lri - 2) * ny + jj]),
                                    R::mul(R::mul(two, d.h1), d.s_hi_neu[j])),
                             three);
}

// V(eval_s, eval_v) by bilinear weights (double result).
template <typename T>
__global__ void k_eval(const T *__restrict__ V, int ny, bilinear b, double *__restrict__ out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const int o = b.i0 * ny + b.j0;
        out[0] = b.w00 * static_cast<double>(V[o]) + b.w10 * static_cast<double>(V[o + ny]) +
                 b.w01 * static_cast<double>(V[o + 1]) + b.w11 * static_cast<double>(V[o + ny + 1]);
    }
}

// ------------------------------------------------------------------------------------------
// Time-dependent coefficients: M, P, Z, C on the grid and D on the v = v_lo line at the time
// of this step (general_heston_equation_coefficients, coefficients.hpp:89-98, on the
// transformed data of lss_heat_data_transform.hpp:174-214), from the time-independent
// factors and this step's D(t) powers da = D^(2(1-beta)), dc = D^(1-beta).
// ------------------------------------------------------------------------------------------
template <typename T> struct time_tables {
    const double *a_static, *c_static; // nx*ny
    const T *ab;                       // nx*ny
    const T *per_i;                    // 5*nx: A, A*A, A*A*A, A', user d
    T *M, *P, *Z, *C, *D0;
    T alpha, delta, two_alpha, half_rho_f;
};

template <typename T, bool X>
__global__ void k_refresh(time_tables<T> tt, int nx, int ny, double da, double dc)
{
    using R = ar<X>;
    const size_t o = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (o >= static_cast<size_t>(nx) * ny) return;
    const int i = static_cast<int>(o / ny), j = static_cast<int>(o % ny);
    const T aval = tt.per_i[i], aa = tt.per_i[nx + i], aaa = tt.per_i[2 * nx + i];
    const T gc = tt.per_i[3 * nx + i], ud = tt.per_i[4 * nx + i];
    const T A = static_cast<T>(__dmul_rn(tt.a_static[o], da));
    const T ah = R::div(A, aa);
    const T ch = R::div(static_cast<T>(__dmul_rn(tt.c_static[o], dc)), tt.ab[o]);
    const T dh = R::sub(R::div(ud, aval), R::div(R::mul(A, gc), aaa));
    const T aah = R::mul(tt.alpha, ah), ddh = R::mul(tt.delta, dh);
    tt.M[o] = R::sub(aah, ddh);
    tt.P[o] = R::add(aah, ddh);
    tt.Z[o] = R::sub(R::mul(tt.two_alpha, ah), tt.half_rho_f);
    tt.C[o] = ch;
    if (j == 0) tt.D0[i] = dh;
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
template <typename T> int plain_solver<T>::init(instance_tables<T> &&tab, int arith, double eval_s, double eval_v)
{
    tab_ = std::move(tab);
    arith_ = arith;
    const int nx = tab_.nx, ny = tab_.ny;
    const size_t n = static_cast<size_t>(nx) * ny;
    // one block of coefficient and boundary tables, or one per step (time-dependent tables)
    const size_t blocks = tab_.step_tables ? static_cast<size_t>(tab_.steps) : 1;
    const size_t sblk = 3 * static_cast<size_t>(nx) + ny + ny + nx;
    LSS_CUDA_TRY(coef_.alloc(7 * n * blocks), "allocating coefficient tables");
    LSS_CUDA_TRY(coef_.upload(tab_.coef.data(), 7 * n * blocks), "uploading coefficient tables");
    LSS_CUDA_TRY(small_.alloc(sblk * blocks), "allocating boundary tables");
    std::vector<T> sm;
    sm.reserve(sblk * blocks);
    for (size_t b = 0; b < blocks; ++b) {
        sm.insert(sm.end(), tab_.coef_v0.begin() + 3 * nx * b, tab_.coef_v0.begin() + 3 * nx * (b + 1));
        sm.insert(sm.end(), tab_.s_lo.begin() + ny * b, tab_.s_lo.begin() + ny * (b + 1));
        sm.insert(sm.end(), tab_.s_hi_neu.begin() + ny * b, tab_.s_hi_neu.begin() + ny * (b + 1));
        sm.insert(sm.end(), tab_.v_hi.begin() + nx * b, tab_.v_hi.begin() + nx * (b + 1));
    }
    LSS_CUDA_TRY(small_.upload(sm.data(), sm.size()), "uploading boundary tables");
    LSS_CUDA_TRY(maps_.alloc(nx + ny), "allocating index maps");
    std::vector<int> mp(tab_.imap);
    mp.insert(mp.end(), tab_.jmap.begin(), tab_.jmap.end());
    LSS_CUDA_TRY(maps_.upload(mp.data(), mp.size()), "uploading index maps");
    // state: U, V, Y1..Y4, G (zero-initialised: rows 0 and nx-1 of Y2 stay zero, as the
    // reference's freshly constructed intermediate containers)
    LSS_CUDA_TRY(state_.alloc(7 * n + 2 * nx), "allocating state");
    LSS_CUDA_TRY(cudaMemset(state_.p, 0, state_.n * sizeof(T)), "clearing state");
    LSS_CUDA_TRY(value_.alloc(1), "allocating value");
    LSS_CUDA_TRY(cudaDeviceSynchronize(), "uploading tables");

    const T *c = coef_.p;
    d_.nx = nx;
    d_.ny = ny;
    d_.theta = tab_.sc.theta;
    d_.zeta = tab_.sc.zeta;
    d_.gamma = tab_.sc.gamma;
    d_.delta = tab_.sc.delta;
    d_.ni = tab_.sc.ni;
    d_.rho = tab_.sc.rho;
    d_.h1 = tab_.sc.h1;
    d_.M = c;
    d_.P = c + n;
    d_.Z = c + 2 * n;
    d_.Mt = c + 3 * n;
    d_.Pt = c + 4 * n;
    d_.W = c + 5 * n;
    d_.C = c + 6 * n;
    d_.D0 = small_.p;
    d_.E0 = small_.p + nx;
    d_.F0 = small_.p + 2 * nx;
    d_.s_lo = small_.p + 3 * nx;
    d_.s_hi_neu = small_.p + 3 * nx + ny;
    d_.v_hi = small_.p + 3 * nx + 2 * ny;
    d_.imap = maps_.p;
    d_.jmap = maps_.p + nx;
    d_.ds = tab_.double_sweep;
    if (tab_.tdep) {
        LSS_CUDA_TRY(tdep_d_.alloc(2 * n), "allocating time-dependent tables");
        LSS_CUDA_TRY(tdep_d_.upload(tab_.a_static.data(), n), "uploading time-dependent tables");
        LSS_CUDA_TRY(cudaMemcpy(tdep_d_.p + n, tab_.c_static.data(), n * sizeof(double), cudaMemcpyHostToDevice),
                     "uploading time-dependent tables");
        LSS_CUDA_TRY(tdep_t_.alloc(n + 5 * static_cast<size_t>(nx)), "allocating time-dependent tables");
        LSS_CUDA_TRY(tdep_t_.upload(tab_.ab.data(), n), "uploading time-dependent tables");
        LSS_CUDA_TRY(cudaMemcpy(tdep_t_.p + n, tab_.per_i.data(), 5 * nx * sizeof(T), cudaMemcpyHostToDevice),
                     "uploading time-dependent tables");
        LSS_CUDA_TRY(cudaDeviceSynchronize(), "uploading time-dependent tables");
    }
    bil_ = make_bilinear(tab_.x.data(), nx, tab_.y.data(), ny, eval_s, eval_v);
    return LSS_ADI_OK;
}

template <typename T> template <bool X> void plain_solver<T>::enqueue_steps(cudaStream_t s, T *&U, T *&V)
{
    const int nx = d_.nx, ny = d_.ny;
    const size_t n = static_cast<size_t>(nx) * ny;
    T *Y1 = state_.p + 2 * n, *Y2 = state_.p + 3 * n, *Y3 = state_.p + 4 * n, *Y4 = state_.p + 5 * n;
    T *G = state_.p + 6 * n, *bcol0 = state_.p + 7 * n, *bcolN = bcol0 + nx;
    const int bs = 64;
    const int gs = grid_for(ny - 2, bs), gv = grid_for(nx - 2, bs);
    const dim3 ghv(grid_for(ny - 2, 128), nx - 2);
    time_tables<T> tt{};
    if (tab_.tdep) {
        tt.a_static = tdep_d_.p;
        tt.c_static = tdep_d_.p + n;
        tt.ab = tdep_t_.p;
        tt.per_i = tdep_t_.p + n;
        tt.M = coef_.p;
        tt.P = coef_.p + n;
        tt.Z = coef_.p + 2 * n;
        tt.C = coef_.p + 6 * n;
        tt.D0 = small_.p;
        tt.alpha = tab_.sc.alpha;
        tt.delta = tab_.sc.delta;
        tt.two_alpha = tab_.two_alpha;
        tt.half_rho_f = tab_.half_rho_f;
    }
    const int gref = grid_for(static_cast<long long>(nx) * ny, 256);
    const size_t sblk = 3 * static_cast<size_t>(nx) + ny + ny + nx;
    for (int step = 0; step < tab_.steps; ++step) {
        // the tables of this step (time-dependent tables: block `step`)
        dev_instance<T> d_ = this->d_;
        if (tab_.step_tables) {
            const size_t oc = 7 * n * static_cast<size_t>(step), os = sblk * static_cast<size_t>(step);
            d_.M += oc; d_.P += oc; d_.Z += oc; d_.Mt += oc; d_.Pt += oc; d_.W += oc; d_.C += oc;
            d_.D0 += os; d_.E0 += os; d_.F0 += os; d_.s_lo += os; d_.s_hi_neu += os; d_.v_hi += os;
        }
        if (tab_.tdep) {
            k_refresh<T, X><<<gref, 256, 0, s>>>(tt, nx, ny, tab_.step_da[step], tab_.step_dc[step]);
            launches_ += 1;
        }
        if (tab_.scheme == LSS_ADI_EXPLICIT_EULER) {
            // heston_euler_time_loop::run: interior, then boundary #1 into columns 0 / ny-1 of
            // the next state, then boundary #2 (its rows 0 / nx-1)
            k_euler<T, X><<<ghv, 128, 0, s>>>(d_, U, V);
            k_boundary1<T, X><<<grid_for(nx, 128), 128, 0, s>>>(d_, U, V, V + (ny - 1), ny);
            k_boundary2<T, X><<<grid_for(ny, 128), 128, 0, s>>>(d_, V);
            launches_ += 3;
            std::swap(U, V);
            continue;
        }
        k_boundary1<T, X><<<grid_for(nx, 128), 128, 0, s>>>(d_, U, bcol0, bcolN, 1);
        k_s_sweep<T, X, S_STAGE1><<<gs, bs, 0, s>>>(d_, U, U, nullptr, nullptr, Y1, G);
        switch (tab_.scheme) {
        case LSS_ADI_DOUGLAS_RACHFORD:
            k_v_sweep<T, X><<<gv, bs, 0, s>>>(d_, U, Y1, bcol0, bcolN, V, G);
            launches_ += 3;
            break;
        case LSS_ADI_CRAIG_SNEYD:
        case LSS_ADI_MODIFIED_CRAIG_SNEYD:
            k_v_sweep<T, X><<<gv, bs, 0, s>>>(d_, U, Y1, bcol0, bcolN, Y2, G);
            if (tab_.scheme == LSS_ADI_CRAIG_SNEYD)
                k_s_sweep<T, X, S_STAGE3_CS><<<gs, bs, 0, s>>>(d_, U, U, Y1, Y2, Y3, G);
            else
                k_s_sweep<T, X, S_STAGE3_MCS><<<gs, bs, 0, s>>>(d_, U, U, Y1, Y2, Y3, G);
            k_v_sweep<T, X><<<gv, bs, 0, s>>>(d_, U, Y3, bcol0, bcolN, V, G);
            launches_ += 5;
            break;
        default: // Hundsdorfer-Verwer
            k_v_sweep<T, X><<<gv, bs, 0, s>>>(d_, U, Y1, bcol0, bcolN, Y2, G);
            k_hv_stage3<T, X><<<ghv, 128, 0, s>>>(d_, U, Y1, Y2, Y3);
            k_s_sweep<T, X, S_STAGE4_HV><<<gs, bs, 0, s>>>(d_, U, Y2, Y3, nullptr, Y4, G);
            k_v_sweep<T, X><<<gv, bs, 0, s>>>(d_, Y2, Y4, bcol0, bcolN, V, G);
            launches_ += 6;
            break;
        }
        k_boundary2<T, X><<<grid_for(ny, 128), 128, 0, s>>>(d_, V);
        launches_ += 1;
        std::swap(U, V);
    }
}

template <typename T>
int plain_solver<T>::forward(const void *payoff, void *out_surface, double *out_value, int flags, void *stream,
                             bool use_graph)
{
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t n = static_cast<size_t>(d_.nx) * d_.ny;
    const bool dev = (flags & LSS_ADI_DEVICE_POINTERS) != 0;
    T *U0 = state_.p, *V0 = state_.p + n;
    const T *src = payoff ? static_cast<const T *>(payoff) : tab_.payoff.data();
    const bool src_dev = payoff && dev;
    LSS_CUDA_TRY(cudaMemcpyAsync(U0, src, n * sizeof(T), src_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s),
                 "copying the terminal condition");
    launches_ = 0;
    T *U = U0, *V = V0;
    if (use_graph) {
        // The loop alternates U/V; capture it once per parity of the step count and replay.
        if (!graph_exec_) {
            cudaStream_t cs;
            LSS_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "creating capture stream");
            LSS_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "beginning graph capture");
            T *u = U0, *v = V0;
            if (arith_ == LSS_ADI_ARITH_REFERENCE)
                enqueue_steps<true>(cs, u, v);
            else
                enqueue_steps<false>(cs, u, v);
            cudaGraph_t g;
            cudaError_t e = cudaStreamEndCapture(cs, &g);
            cudaStreamDestroy(cs);
            LSS_CUDA_TRY(e, "ending graph capture");
            e = cudaGraphInstantiate(&graph_exec_, g, 0);
            cudaGraphDestroy(g);
            LSS_CUDA_TRY(e, "instantiating graph");
            graph_launches_ = launches_;
        }
        LSS_CUDA_TRY(cudaGraphLaunch(graph_exec_, s), "launching graph");
        launches_ = graph_launches_;
        if (tab_.steps % 2) std::swap(U, V);
    } else {
        if (arith_ == LSS_ADI_ARITH_REFERENCE)
            enqueue_steps<true>(s, U, V);
        else
            enqueue_steps<false>(s, U, V);
    }
    LSS_CUDA_TRY(cudaGetLastError(), "launching the time loop");
    if (out_value) {
        k_eval<T><<<1, 32, 0, s>>>(U, d_.ny, bil_, value_.p);
        ++launches_;
        LSS_CUDA_TRY(cudaGetLastError(), "launching k_eval");
        LSS_CUDA_TRY(cudaMemcpyAsync(out_value, value_.p, sizeof(double), cudaMemcpyDeviceToHost, s), "reading value");
    }
    if (out_surface) {
        LSS_CUDA_TRY(cudaMemcpyAsync(out_surface, U, n * sizeof(T), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s),
                     "copying the surface");
    }
    if (!dev || out_value) LSS_CUDA_TRY(cudaStreamSynchronize(s), "running the time loop");
    return LSS_ADI_OK;
}

template <typename T> plain_solver<T>::~plain_solver()
{
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
}

template struct plain_solver<double>;
template struct plain_solver<float>;

} // namespace lss_gb300
