// adi_adjoint.cuh -- reverse-mode (adjoint) of one ADI time step in the factorised form
// used by the batched kernel, for Douglas-Rachford, Craig-Sneyd, modified Craig-Sneyd and
// Hundsdorfer-Verwer.
//
// Forward step (see adi_batched.cu): B1 -> S1 -> V1 -> S2 -> V2 -> B2, where each S/V stage
// solves  a x_{t-1} + b x_t + c x_{t+1} = f_t  per line through the precomputed factors
//   y_t = f_t/beta_t - la_t y_{t-1},   x_t = y_t - g_t x_{t+1}   (y_0 = lo, x_{e+1} = hi).
// The adjoint of such a solve, given xbar_t, is
//   z_t = xbar_t - g_{t-1} z_{t-1}          (t = 1..e)
//   w_t = z_t - la_{t+1} w_{t+1}            (t = e..1)
//   fbar_t(scaled) = w_t,  lobar = -la_1 w_1,  hibar = -ch w_e,
// i.e. the transposed factorisation, one FMA per point each way.  Right-hand-side terms
// that stay on the line are applied by the line's thread; cross-line terms (mixed
// derivative, neighbouring lines) by a gather pass over columns.  Parameter
// sensitivities dV/d(kappa, theta, sigma, rho, r) use, per stage and grid point,
//   mu_t * (d f_t/dp - d a_t/dp x_{t-1} - d b_t/dp x_t - d c_t/dp x_{t+1}),  mu_t = w_t / beta_t,
// with the coefficient derivatives of the model (Heston, or SABR at r = 0 whose D(t) terms add
// a per-step factor tau = T - t), all separable into 1-D tables.
#pragma once
// Included by adi_batched.cu inside namespace lss_gb300, after the forward stage functions.

struct adj_acc {
    // S-line sums, already scaled: r, kappa, theta, sigma, rho
    double s[5];
    // v-line raw sums: sum mu (dm-dn) ek, (dm-dn) et, (dm-dn) es, (2dc-dm-dn) bs, dc
    double vk, vt, vs1, vs2, vb;
};

// B2^T: fold the S_max extrapolation row into rows nx-2 / nx-3; clear rows 0 and nx-1 of UB
// (all of UB for Hundsdorfer-Verwer, whose last v stage feeds Y2B instead of UB).
__device__ __forceinline__ void adj_b2(const inst_view<double> &v, double *__restrict__ VB, double *__restrict__ UB,
                                       bool clear_all, int l0, int ls)
{
    const int nx = v.nx, ny = v.ny, lri = nx - 1;
    const double four3 = 4.0 / 3.0, third = 1.0 / 3.0;
    for (int q = l0; q < ny; q += ls) {
        double add = 0.0;
        if (__ldg(v.jmap() + q) == q) add += VB[(long long)lri * ny + q];
        if (q + 1 < ny && __ldg(v.jmap() + q + 1) == q) add += VB[(long long)lri * ny + q + 1];
        VB[(long long)(lri - 1) * ny + q] += four3 * add;
        VB[(long long)(lri - 2) * ny + q] -= third * add;
        if (clear_all) {
            for (int p = 0; p < nx; ++p) UB[(long long)p * ny + q] = 0.0;
        } else {
            UB[q] = 0.0;
            UB[(long long)lri * ny + q] = 0.0;
        }
    }
}

// Parameter sums of one v-line point: mu = ib * w, dm / dc / dn = (in - out) at t-1, t, t+1.
__device__ __forceinline__ void adj_v_sum(const inst_view<double> &v, int t, double mu, double dm, double dc, double dn,
                                          adj_acc &acc)
{
    const double q = mu * (dm - dn);
    acc.vk += q * __ldg(v.Yv(Y_EK) + t);
    acc.vt += q * __ldg(v.Yv(Y_ET) + t);
    acc.vs1 += q * __ldg(v.Yv(Y_ES) + t);
    acc.vs2 += mu * (2.0 * dc - dm - dn) * __ldg(v.Yv(Y_BS) + t);
    acc.vb += mu * dc;
}

// V-line stage adjoint.  XB: adjoint of the stage output (rows i, incl. the lo copy at t=0);
// in/out: the stage's `in` array and its output; INB (+)= adjoint of `in`; INHB (+)= adjoint
// of `inh`; LV (+)= adjoint of the line's lo value.
template <bool FIRST>
__device__ __forceinline__ void adj_v(const inst_view<double> &v, const double *__restrict__ in,
                                      const double *__restrict__ out, const double *__restrict__ XB,
                                      double *__restrict__ INB, double *__restrict__ INHB, double *__restrict__ TMP,
                                      double *__restrict__ LV, adj_acc &acc, int l0, int ls)
{
    const int nx = v.nx, ny = v.ny, e = ny - 2;
    for (int i = 1 + l0; i <= nx - 2; i += ls) {
        const long long row = (long long)i * ny;
        double z = 0.0;
#pragma unroll 4
        for (int t = 1; t <= e; ++t) {
            const double gprev = (t > 1) ? __ldg(v.Vt(VL_G) + (long long)(t - 1) * nx + i) : 0.0;
            z = XB[row + t] - gprev * z;
            TMP[row + t] = z;
        }
        double w = 0.0, la_next = 0.0;
        double acc_t1 = 0.0, acc_t = 0.0; // pending adjoint of in(t+1) / in(t)
        // windows of (in - out) at t+1 and t
        double dn = in[row + e + 1] - out[row + e + 1];
        double dc = in[row + e] - out[row + e];
#pragma unroll 4
        for (int t = e; t >= 1; --t) {
            const long long ot = (long long)t * nx + i;
            w = TMP[row + t] - la_next * w;
            const double la = __ldg(v.Vt(VL_LA) + ot), vc = __ldg(v.Vt(VL_VC) + ot), vn = __ldg(v.Vt(VL_VN) + ot);
            const double ib = __ldg(v.Vt(VL_IB) + ot);
            const double fin = acc_t1 + vn * w; // adjoint of in(t+1) is complete
            if (FIRST) INB[row + t + 1] = fin; else INB[row + t + 1] += fin;
            acc_t1 = acc_t + vc * w;
            acc_t = la * w;
            const double mu = ib * w;
            if (FIRST) INHB[row + t] = mu; else INHB[row + t] += mu;
            const double dm = in[row + t - 1] - out[row + t - 1];
            adj_v_sum(v, t, mu, dm, dc, dn, acc);
            dn = dc;
            dc = dm;
            la_next = la;
        }
        if (FIRST) { INB[row + 1] = acc_t1; INB[row] = acc_t; }
        else { INB[row + 1] += acc_t1; INB[row] += acc_t; }
        const double lob = -la_next * w + XB[row];
        if (FIRST) LV[i] = lob; else LV[i] += lob;
    }
}

// Line sums of mu * d(residual)/d(parameter) pieces of an S line (the S-direction factors of the
// coefficient derivatives applied per point; the v-direction ones once per line, adj_s_line).
// The stage's constant factors (theta, the Delta weight, gamma, zeta gamma) are taken out of the
// per-point work: the second S stage keeps the theta parts (A, B, Aa, Dd) and the Delta parts
// (A2, B2, Aa2, Dd2, Q, D) apart and adj_s_line weighs them once per line.
struct s_sums {
    double A, A2, B, B2, Q, D, E, Aa, Aa2, Dd, Dd2;
};
// Per point, mu times the coefficient derivatives of the stage residual (d/dM, d/dZ, d/dP,
// d/dM~, d/dW, d/dP~, d/dC) enter the parameter sums only as P - M, Z + W, P~ - M~,
// M~ + P~ + 2W, C and M + P + 2Z: a three-row window along the line (rows t+1, t, t-1, one new
// row per point; adj_s_row) gives them from per-row quantities
//   KIND 1 (first S stage, output Yo = Y1): f = (1-theta) U + theta Yo, c = U, s / n = U at
//          j-1 / j+1, dd = s - n;
//   KIND 2 (second S stage of CS/MCS/HV): the same on Delta = Y2 - U, with f = Yo - U
//          (CS/MCS) or Yo - Y1 - Delta (HV).
struct s_row {
    double f, c, s, n, dd;
};
template <int KIND, int SCH>
__device__ __forceinline__ s_row adj_s_row(const double *__restrict__ U, const double *__restrict__ Y1,
                                           const double *__restrict__ Y2, const double *__restrict__ Yo, long long q,
                                           double th, double omth)
{
    s_row w;
    if constexpr (KIND == 1) {
        w.s = U[q - 1];
        w.c = U[q];
        w.n = U[q + 1];
        w.f = omth * w.c + th * Yo[q];
    } else {
        w.s = Y2[q - 1] - U[q - 1];
        w.c = Y2[q] - U[q];
        w.n = Y2[q + 1] - U[q + 1];
        w.f = SCH == LSS_ADI_HUNDSDORFER_VERWER ? (Yo[q] - Y1[q] - w.c) : (Yo[q] - U[q]);
    }
    w.dd = w.s - w.n;
    return w;
}
// Weight of the Delta = Y2 - U terms of the second S stage: zeta - theta for MCS (with the
// reference's sign of the P term), zeta for HV (textbook sign), none for CS.
template <int SCH> __device__ __forceinline__ double delta_weight(const bdesc &d)
{
    return SCH == LSS_ADI_MODIFIED_CRAIG_SNEYD ? d.a_zeta - d.a_theta
                                               : SCH == LSS_ADI_HUNDSDORFER_VERWER ? d.a_zeta : 0.0;
}
// Sums of one point from the rows t+1 (rh), t (rc), t-1 (rl); muX = mu (S/A)(t), muC = mu times
// the S factor of c^ (the same table for Heston).
template <int KIND, int SCH>
__device__ __forceinline__ void adj_s_point(const inst_view<double> &v, s_sums &p, const s_row &rh, const s_row &rc,
                                            const s_row &rl, double mu, double muX, double muC, int t, bool sabr)
{
    constexpr bool xt = KIND == 2 && (SCH == LSS_ADI_MODIFIED_CRAIG_SNEYD || SCH == LSS_ADI_HUNDSDORFER_VERWER);
    constexpr double sp = SCH == LSS_ADI_HUNDSDORFER_VERWER ? 1.0 : -1.0;
    const double PmM = rh.f - rl.f;
    p.A += muX * PmM;
    if constexpr (KIND == 1)
        p.B -= mu * (rc.f + rc.c);
    else
        p.B -= mu * rc.f;
    p.E += muC * (rl.dd - rh.dd);
    if constexpr (KIND == 1 || xt) {
        p.Q -= mu * rc.dd;
        p.D += mu * (rc.s + rc.n - 2.0 * rc.c);
    }
    double PmM2 = 0.0;
    if constexpr (xt) {
        PmM2 = sp * rh.c - rl.c;
        p.A2 += muX * PmM2;
        p.B2 -= mu * rc.c;
    }
    if (sabr) {
        const double ha = mu * __ldg(v.X(X_HA) + t), hd = mu * __ldg(v.X(X_HDD) + t);
        p.Aa += ha * (rl.f + rh.f - 2.0 * rc.f);
        p.Dd += hd * PmM;
        if constexpr (xt) {
            p.Aa2 += ha * (rl.c + sp * rh.c - 2.0 * rc.c);
            p.Dd2 += hd * PmM2;
        }
    }
}
// The line's sums, weighed by the stage's constants and the v-direction factors of the line.
template <int KIND, int SCH>
__device__ __forceinline__ void adj_s_line(const inst_view<double> &v, const bdesc &d, int j, const s_sums &p,
                                           double tau, bool sabr, adj_acc &acc)
{
    double A, B, Q, D, E, Aa, Dd;
    if constexpr (KIND == 1) {
        A = p.A;
        B = p.B;
        Q = p.Q;
        D = p.D;
        E = d.a_gamma * p.E;
        Aa = p.Aa;
        Dd = p.Dd;
    } else {
        const double th = d.a_theta, zt = delta_weight<SCH>(d);
        A = th * p.A + zt * p.A2;
        B = th * p.B + 2.0 * zt * p.B2;
        Q = zt * p.Q;
        D = zt * p.D;
        E = d.a_zeta * d.a_gamma * p.E;
        Aa = th * p.Aa + zt * p.Aa2;
        Dd = th * p.Dd + zt * p.Dd2;
    }
    const double ek = __ldg(v.Yv(Y_EK) + j), et = __ldg(v.Yv(Y_ET) + j), es = __ldg(v.Yv(Y_ES) + j);
    const double bs = __ldg(v.Yv(Y_BS) + j), hy = __ldg(v.Yv(Y_HY) + j);
    acc.s[0] += d.a_delta * A + d.a_halfk * B;
    if (sabr) // D(t) terms of a^, d^ and c^
        acc.s[0] += tau * d.a_omb *
                    (__ldg(v.Yv(Y_HV2) + j) * (2.0 * d.a_delta * Dd - 2.0 * d.a_alphat * Aa) - d.a_rho * d.a_sigma * hy * E);
    acc.s[1] += d.a_ni * ek * Q;
    acc.s[2] += d.a_ni * et * Q;
    acc.s[3] += d.a_ni * es * Q + d.a_betat * bs * D + d.a_rho * hy * E;
    acc.s[4] += d.a_sigma * hy * E;
}

// S-line stage adjoint.  KIND 1: S1 (explicit operator on U, output Y1).  KIND 2: second S
// stage of CS/MCS/HV (output Y3).  XB: adjoint of the stage output; FB receives the scaled
// right-hand-side adjoint w; LS/HS the lo/hi adjoints of the line.  The along-line terms of
// the second stage act on U for CS/MCS and on Y1 for HV, whose right-hand side is
// (I - theta k A1) Y1 + (zeta k A - theta k A1)(Y2 - U) (hundsdorfer_verwer_method.hpp:128-194).
template <int KIND, int SCH>
__device__ __forceinline__ void adj_s(const inst_view<double> &v, const bdesc &d, const double *__restrict__ U,
                                      const double *__restrict__ Y1, const double *__restrict__ Y2,
                                      const double *__restrict__ Yo, const double *__restrict__ XB,
                                      double *__restrict__ FB, double *__restrict__ TMP, double *__restrict__ LS,
                                      double *__restrict__ HS, double *__restrict__ UB, double *__restrict__ Y1B,
                                      adj_acc &acc, double tau, int l0, int ls)
{
    constexpr bool hv = SCH == LSS_ADI_HUNDSDORFER_VERWER;
    const int nx = v.nx, ny = v.ny, e = nx - 2;
    const bool sabr = d.model == LSS_ADI_SABR;
    const double th = d.a_theta, omth = 1.0 - d.a_theta;
    for (int j = 1 + l0; j <= ny - 2; j += ls) {
        double z = 0.0;
#pragma unroll 4
        for (int t = 1; t <= e; ++t) {
            const long long o = (long long)t * ny + j;
            const double gprev = (t > 1) ? __ldg(v.S(SL_G) + o - ny) : 0.0;
            z = XB[o] - gprev * z;
            TMP[o] = z;
        }
        double w = 0.0, la_next = 0.0, w_e = 0.0;
        double acc_t1 = 0.0, acc_t = 0.0;
        s_sums ps = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        // three-row window along the line (rows t+1, t, t-1; one new row per point)
        auto load_row = [&](int r) -> s_row { return adj_s_row<KIND, SCH>(U, Y1, Y2, Yo, (long long)r * ny + j, th, omth); };
        s_row rh = load_row(e + 1), rc = load_row(e);
#pragma unroll 2
        for (int t = e; t >= 1; --t) {
            const long long o = (long long)t * ny + j;
            const s_row rl = load_row(t - 1);
            w = TMP[o] - la_next * w;
            if (t == e) w_e = w;
            FB[o] = w;
            const double la = __ldg(v.S(SL_LA) + o);
            const double mu = __ldg(v.S(SL_IB) + o) * w;
            if constexpr (KIND == 2) {
                // along-line terms of the second S stage: la A(t-1) + sc A(t) + se A(t+1) (+ ib Y1(t)),
                // A = U for CS/MCS, A = Y1 for HV (its rows are written once here: no accumulation)
                const double sc = __ldg(v.S(SL_S2SC) + o), se = __ldg(v.S(SL_S2SE) + o);
                const double fin = acc_t1 + se * w;
                acc_t1 = acc_t + sc * w;
                acc_t = la * w;
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
            la_next = la;
            rh = rc;
            rc = rl;
        }
        if constexpr (KIND == 2) {
            if constexpr (hv) {
                Y1B[(long long)ny + j] = acc_t1;
                Y1B[j] = acc_t;
            } else {
                UB[(long long)ny + j] += acc_t1;
                UB[j] += acc_t;
            }
        }
        LS[j] = -la_next * w + XB[j];
        HS[j] = -__ldg(v.Yv(Y_CHS) + j) * w_e + XB[(long long)(nx - 1) * ny + j];
        adj_s_line<KIND, SCH>(v, d, j, ps, tau, sabr, acc);
    }
}

// B1^T at grid point (p, q <= 2): the adjoint of the explicit v = v_lo boundary column, whose
// values are the lo ends of the v lines (bbar0(i) = sum of LV over lines i' with imap[i'] = i),
// with its parameter sensitivities (D, E, F of the v = v_lo line) at q = 0.
__device__ __forceinline__ double adj_b1_terms(const inst_view<double> &v, const bdesc &d, const double *__restrict__ U,
                                               const double *__restrict__ LV, adj_acc &acc, double tau, int p, int q)
{
    const int nx = v.nx, ny = v.ny;
    auto B0 = [&](int i) -> double {
        if (i < 1 || i > nx - 2) return 0.0;
        double sum = 0.0;
        if (__ldg(v.imap() + i) == i) sum += LV[i];
        if (i + 1 <= nx - 2 && __ldg(v.imap() + i + 1) == i) sum += LV[i + 1];
        return sum;
    };
    const long long o = (long long)p * ny + q;
    if (q == 1) return __ldg(v.X(XB_1) + p) * B0(p);
    if (q == 2) return __ldg(v.X(XB_2) + p) * B0(p);
    const double val = (p + 1 <= nx - 2 ? __ldg(v.X(XB_M) + p + 1) * B0(p + 1) : 0.0) + __ldg(v.X(XB_C) + p) * B0(p) +
                       (p >= 1 ? __ldg(v.X(XB_P) + p - 1) * B0(p - 1) : 0.0);
    if (p >= 1 && p <= nx - 2) {
        const double bb = B0(p);
        if (bb != 0.0) {
            const double u0 = U[o], u1 = U[o + 1], u2 = U[o + 2];
            const double um = U[o - ny], up = U[o + ny];
            const double ee = d.a_ni * bb * (4.0 * u1 - 3.0 * u0 - u2);
            double hd = __ldg(v.X(X_HX) + p);
            if (d.model == LSS_ADI_SABR) hd += 2.0 * d.a_omb * tau * __ldg(v.Yv(Y_HV2)) * __ldg(v.X(X_HDD) + p);
            acc.s[0] += bb * (d.a_delta * hd * (up - um) - d.a_k * u0);
            acc.s[1] += ee * __ldg(v.Yv(Y_EK));
            acc.s[2] += ee * __ldg(v.Yv(Y_ET));
            acc.s[3] += ee * __ldg(v.Yv(Y_ES));
        }
    }
    return val;
}

// Gather: cross-line right-hand-side adjoints of an S stage into UB (and Y2B for KIND 2), the
// lo/hi adjoints of the S lines (lsum / hsum of column q, added on rows 0 / nx-1), and for
// KIND 1 the adjoint of the explicit v = v_lo boundary column (B1^T) with its parameter
// sensitivities.  One grid point (p, q) per call.
template <int KIND>
__device__ __forceinline__ void adj_gather_point(const inst_view<double> &v, const bdesc &d, const double *__restrict__ U,
                                                 const double *__restrict__ FB, const double *__restrict__ LV,
                                                 double *__restrict__ UB, double *__restrict__ Y2B, adj_acc &acc,
                                                 double tau, int p, int q, double lsum, double hsum)
{
    const int nx = v.nx, ny = v.ny;
    auto F = [&](int a, int b) -> double {
        return (a >= 1 && a <= nx - 2 && b >= 1 && b <= ny - 2) ? FB[(long long)a * ny + b] : 0.0;
    };
    auto W = [&](int slot, int a, int b) -> double {
        return (a >= 1 && a <= nx - 2 && b >= 1 && b <= ny - 2) ? __ldg(v.S(slot) + (long long)a * ny + b) : 0.0;
    };
    const long long o = (long long)p * ny + q;
    double val = 0.0;
    if constexpr (KIND == 2) {
        double db = W(SL_S2MZ, p + 1, q + 1) * F(p + 1, q + 1) - W(SL_S2MZ, p + 1, q - 1) * F(p + 1, q - 1) -
                    W(SL_S2MZ, p - 1, q + 1) * F(p - 1, q + 1) + W(SL_S2MZ, p - 1, q - 1) * F(p - 1, q - 1);
        if (d.scheme != LSS_ADI_CRAIG_SNEYD)
            db += W(SL_X1, p + 1, q) * F(p + 1, q) + W(SL_X2, p, q) * F(p, q) + W(SL_X3, p - 1, q) * F(p - 1, q) +
                  W(SL_X4, p, q + 1) * F(p, q + 1) + W(SL_X5, p, q - 1) * F(p, q - 1);
        // HV: rows 1..nx-2 already hold the last v stage's adjoint of its input Y2
        if (d.scheme == LSS_ADI_HUNDSDORFER_VERWER && p >= 1 && p <= nx - 2) Y2B[o] += db; else Y2B[o] = db;
        val -= db;
    } else {
        val += W(SL_WW, p + 1, q) * F(p + 1, q) + W(SL_WE, p - 1, q) * F(p - 1, q) + W(SL_WS, p, q + 1) * F(p, q + 1) +
               W(SL_WN, p, q - 1) * F(p, q - 1) + W(SL_WC, p, q) * F(p, q) + W(SL_WG, p + 1, q + 1) * F(p + 1, q + 1) -
               W(SL_WG, p + 1, q - 1) * F(p + 1, q - 1) - W(SL_WG, p - 1, q + 1) * F(p - 1, q + 1) +
               W(SL_WG, p - 1, q - 1) * F(p - 1, q - 1);
        if (q <= 2) val += adj_b1_terms(v, d, U, LV, acc, tau, p, q);
    }
    if (p == 0) val += lsum;
    if (p == nx - 1) val += hsum;
    UB[o] += val;
}

// lo / hi adjoints of the S lines whose Dirichlet values come from column q (index_of remap)
__device__ __forceinline__ void adj_line_ends(const inst_view<double> &v, const double *__restrict__ LS,
                                              const double *__restrict__ HS, int q, double &lsum, double &hsum)
{
    const int ny = v.ny;
    lsum = 0.0;
    hsum = 0.0;
    if (q >= 1 && q <= ny - 2 && __ldg(v.jmap() + q) == q) { lsum += LS[q]; hsum += HS[q]; }
    if (q + 1 <= ny - 2 && __ldg(v.jmap() + q + 1) == q) { lsum += LS[q + 1]; hsum += HS[q + 1]; }
}

// Gather pass over columns q (thread per column), walking down the column with a window of three
// rows.  The transposed stencil at (p, q) is  down(p+1) + up(p-1) + mid(p)  where each row r
// contributes, from FB and the weight tables at columns q-1, q, q+1 of that row,
//   KIND 1:  down = WW F + g,  up = WE F - g,  mid = WS(q+1) F(q+1) + WN(q-1) F(q-1) + WC F
//            with g = WG(q+1) F(q+1) - WG(q-1) F(q-1)   (mixed term of the explicit operator);
//   KIND 2:  the same with S2MZ for WG and, for MCS/HV, X1 / X3 / X2, X4, X5 for WW / WE / WC, WS,
//            WN; for CS only the mixed term: down = g, up = -g, mid = 0.
// FB and the tables are zero on the boundary rows and columns of an instance (never written), so
// only the rows and columns outside the instance need guards.  Each row's table and FB values are
// loaded once instead of once per neighbour.
template <int KIND, int SCH>
__device__ __forceinline__ void adj_gather(const inst_view<double> &v, const bdesc &d, const double *__restrict__ U,
                                           const double *__restrict__ FB, const double *__restrict__ LS,
                                           const double *__restrict__ HS, const double *__restrict__ LV,
                                           double *__restrict__ UB, double *__restrict__ Y2B, adj_acc &acc, double tau,
                                           int l0, int ls)
{
    const int nx = v.nx, ny = v.ny;
    constexpr bool xterms = KIND == 1 || SCH != LSS_ADI_CRAIG_SNEYD;
    constexpr bool hv = SCH == LSS_ADI_HUNDSDORFER_VERWER;
    const double *WG = v.S(KIND == 1 ? SL_WG : SL_S2MZ);
    const double *WD = v.S(KIND == 1 ? SL_WW : SL_X1), *WU = v.S(KIND == 1 ? SL_WE : SL_X3);
    const double *WM = v.S(KIND == 1 ? SL_WC : SL_X2), *WR = v.S(KIND == 1 ? SL_WS : SL_X4);
    const double *WL = v.S(KIND == 1 ? SL_WN : SL_X5);
    for (int q = l0; q < ny; q += ls) {
        double lsum, hsum;
        adj_line_ends(v, LS, HS, q, lsum, hsum);
        const bool ql = q >= 1, qr = q + 1 <= ny - 1;
        // row r: its down term dn (used at row r-1), up term (used at row r+1) and mid (row r)
        auto row = [&](int r, double &dn, double &up, double &mid) {
            if (r < 0 || r > nx - 1) {
                dn = up = mid = 0.0;
                return;
            }
            const long long o = (long long)r * ny + q;
            const double f0 = FB[o], fm = ql ? FB[o - 1] : 0.0, fp = qr ? FB[o + 1] : 0.0;
            const double gm = ql ? __ldg(WG + o - 1) * fm : 0.0;
            const double g = qr ? fma(__ldg(WG + o + 1), fp, -gm) : -gm;
            if constexpr (xterms) {
                dn = fma(__ldg(WD + o), f0, g);
                up = fma(__ldg(WU + o), f0, -g);
                mid = (qr ? __ldg(WR + o + 1) * fp : 0.0) + (ql ? __ldg(WL + o - 1) * fm : 0.0) + __ldg(WM + o) * f0;
            } else {
                dn = g;
                up = -g;
                mid = 0.0;
            }
        };
        double up_m = 0.0;          // up of row p-1 (no row above row 0)
        double dn_c, up_c, mid_c;   // row p (its down term is used one row earlier)
        double dn_p, up_p, mid_p;   // row p+1
        row(0, dn_c, up_c, mid_c);
#pragma unroll 2
        for (int p = 0; p < nx; ++p) {
            row(p + 1, dn_p, up_p, mid_p);
            const long long o = (long long)p * ny + q;
            double val;
            if constexpr (KIND == 2) {
                const double db = xterms ? dn_p + up_m + mid_c : dn_p + up_m;
                // HV: rows 1..nx-2 already hold the last v stage's adjoint of its input Y2
                if (hv && p >= 1 && p <= nx - 2) Y2B[o] += db; else Y2B[o] = db;
                val = -db;
            } else {
                val = dn_p + up_m + mid_c; // the B1^T terms of columns 0..2 follow in adj_b1_pass
            }
            if (p == 0) val += lsum;
            if (p == nx - 1) val += hsum;
            UB[o] += val;
            up_m = up_c;
            up_c = up_p;
            mid_c = mid_p;
        }
    }
}

// B1^T terms of columns 0..2 (adj_b1_terms), spread over the CTA's threads by row after the
// column walk of adj_gather<1> (which would otherwise leave the threads of columns 0..2 walking
// their columns alone with this extra work, the rest of their warp idle).
__device__ __forceinline__ void adj_b1_pass(const inst_view<double> &v, const bdesc &d, const double *__restrict__ U,
                                            const double *__restrict__ LV, double *__restrict__ UB, adj_acc &acc,
                                            double tau, int l0, int ls)
{
    const int nx = v.nx, ny = v.ny;
    const int qn = ny < 3 ? ny : 3;
    for (int p = l0; p < nx; p += ls)
        for (int q = 0; q < qn; ++q) UB[(long long)p * ny + q] += adj_b1_terms(v, d, U, LV, acc, tau, p, q);
}

// Adjoint of one time step of scheme SCH: VB = adjoint of the step output (modified in place),
// UB receives the adjoint of the step input.  U/Y1/Y2/Y3/Vo: the step's input, stage outputs and
// output.  Work split over the threads of group g, group barriers between the stages.
template <int SCH>
__device__ __forceinline__ void adj_step(const inst_view<double> &v, const bdesc &d, const double *U, const double *Y1,
                                         const double *Y2, const double *Y3, const double *Vo, double *VB, double *UB,
                                         double *Y1B, double *Y2B, double *Y3B, double *FB, double *TMP, double *LV,
                                         double *LS, double *HS, adj_acc &acc, double tau, const grp &g)
{
    const int l0 = g.t, ls = g.n;
    constexpr bool hv = SCH == LSS_ADI_HUNDSDORFER_VERWER;
    adj_b2(v, VB, UB, hv, l0, ls);
    g.sync();
    if constexpr (SCH == LSS_ADI_DOUGLAS_RACHFORD) {
        adj_v<true>(v, U, Vo, VB, UB, Y1B, TMP, LV, acc, l0, ls);
        g.sync();
    } else {
        // last v stage: in = U (CS/MCS) or Y2 (HV)
        if constexpr (hv)
            adj_v<true>(v, Y2, Vo, VB, Y2B, Y3B, TMP, LV, acc, l0, ls);
        else
            adj_v<true>(v, U, Vo, VB, UB, Y3B, TMP, LV, acc, l0, ls);
        g.sync();
        adj_s<2, SCH>(v, d, U, Y1, Y2, Y3, Y3B, FB, TMP, LS, HS, UB, Y1B, acc, tau, l0, ls);
        g.sync();
        adj_gather<2, SCH>(v, d, U, FB, LS, HS, LV, UB, Y2B, acc, tau, l0, ls);
        g.sync();
        adj_v<false>(v, U, Y2, Y2B, UB, Y1B, TMP, LV, acc, l0, ls);
        g.sync();
    }
    adj_s<1, SCH>(v, d, U, Y1, Y2, Y1, Y1B, FB, TMP, LS, HS, UB, Y1B, acc, tau, l0, ls);
    g.sync();
    adj_gather<1, SCH>(v, d, U, FB, LS, HS, LV, UB, Y2B, acc, tau, l0, ls);
    g.sync();
    adj_b1_pass(v, d, U, LV, UB, acc, tau, l0, ls);
    g.sync();
}
