// Device helpers shared by the assembly and MD-force kernels: the Chebyshev basis
// of one pair distance and the smooth cut-off.
//
// Reference: Cheby::set_polys / set_polys_out_of_range (src/Cheby.C:207-443),
// Cheby::transform / cheby_var_deriv (src/Cheby.C:58-165), FCUT::get_fcut
// (src/Fcut.C:17-72).
#pragma once
#include "dev.cuh"

namespace cgd {

static constexpr double PI_REF = 3.14159265359;   // src/functions.h:48

// ---------------------------------------------------------------- basis
// Cheby::set_polys and set_polys_out_of_range (src/Cheby.C:207-443) evaluated as one
// forward recursion: T_n(x) and U_{n-1}(x) give T'_n = n (dx/dr) U_{n-1}.  Writes
// g[k] = f T_{n0+k} and h[k] = f T'_{n0+k} + f' T_{n0+k} for k < count (stride apart),
// so nothing is kept in local memory.
template <typename Out>
__device__ __forceinline__ void basis_gh(const ModelDev& M, double lambda, double xavg, double xdiff, double smin,
                                         double r, int n0, int count, double fc, double fd, Out* g, Out* h,
                                         int stride) {
    const bool out = r < smin;
    const double rr = out ? smin : r;
    double x, ex = 0.0;
    const double ixd = 1.0 / xdiff;
    if (M.trans == 0) { ex = exp(-rr / lambda); x = (ex - xavg) * ixd; }
    else if (M.trans == 1) { x = (1.0 / rr - xavg) * ixd; }
    else { x = (rr - xavg) * ixd; }
    double dxdr;
    if (M.trans == 0) dxdr = -ex / lambda * ixd;
    else if (M.trans == 1) dxdr = -ixd / (rr * rr);
    else dxdr = ixd;
    dxdr *= M.deriv_const;
    const bool zero_d = out && M.fix == 1;           // ZERO_DERIV
    double damp = 1.0, shift = 0.0;                  // SMOOTH: T += s (damp-1) T', T' *= damp
    if (out && M.fix == 0) { damp = exp((r - smin) / M.smooth); shift = M.smooth * (damp - 1.0); }
    const double lin = (out && M.fix == 2) ? (r - smin) : 0.0;   // CONSTANT_DERIV: T += T' (r - smin)
    double t_prev = 1.0, t_cur = x;          // T_0, T_1
    double u_prev2 = 0.0, u_prev = 1.0;      // U_{-1} (unused), U_0
    const int n1 = n0 + count;
    for (int n = 0; n < n1; ++n) {
        double tn, un_1;                     // T_n, U_{n-1}
        if (n == 0) { tn = 1.0; un_1 = 0.0; }
        else if (n == 1) { tn = x; un_1 = 1.0; }
        else {
            tn = 2.0 * x * t_cur - t_prev;
            t_prev = t_cur; t_cur = tn;
            const double un = (n - 1 == 1) ? 2.0 * x : 2.0 * x * u_prev - u_prev2;   // U_{n-1}
            u_prev2 = u_prev; u_prev = un;
            un_1 = un;
        }
        double td = (n == 0 || zero_d) ? 0.0 : n * dxdr * un_1;
        if (out) {
            if (M.fix == 0) { tn += shift * td; td *= damp; }
            else if (M.fix == 2) tn += td * lin;
        }
        if (n >= n0) {
            g[(n - n0) * stride] = Out(fc * tn);
            h[(n - n0) * stride] = Out(fc * td + fd * tn);
        }
    }
}

// basis_gh with the recursion in the compute type T: the argument x, dx/dr and the
// out-of-range factors are formed in FP64 (one exp per edge), the per-power
// recursion and products in T.  For T = double this is basis_gh itself.
template <typename T>
__device__ __forceinline__ void basis_gh_t(const ModelDev& M, double lambda, double xavg, double xdiff, double smin,
                                           double r, int n0, int count, double fc, double fd, T* g, T* h,
                                           int stride) {
    if constexpr (sizeof(T) == 8) {
        basis_gh(M, lambda, xavg, xdiff, smin, r, n0, count, fc, fd, g, h, stride);
    } else {
        const bool out = r < smin;
        const double rr = out ? smin : r;
        double xd, ex = 0.0;
        const double ixd = 1.0 / xdiff;
        if (M.trans == 0) { ex = exp(-rr / lambda); xd = (ex - xavg) * ixd; }
        else if (M.trans == 1) { xd = (1.0 / rr - xavg) * ixd; }
        else { xd = (rr - xavg) * ixd; }
        double dxdr_d;
        if (M.trans == 0) dxdr_d = -ex / lambda * ixd;
        else if (M.trans == 1) dxdr_d = -ixd / (rr * rr);
        else dxdr_d = ixd;
        dxdr_d *= M.deriv_const;
        const bool zero_d = out && M.fix == 1;
        double damp_d = 1.0, shift_d = 0.0;
        if (out && M.fix == 0) { damp_d = exp((r - smin) / M.smooth); shift_d = M.smooth * (damp_d - 1.0); }
        const T x = T(xd), dxdr = T(dxdr_d), damp = T(damp_d), shift = T(shift_d);
        const T lin = T((out && M.fix == 2) ? (r - smin) : 0.0);
        const T tfc = T(fc), tfd = T(fd);
        T t_prev = T(1), t_cur = x, u_prev2 = T(0), u_prev = T(1);
        const int n1 = n0 + count;
        for (int n = 0; n < n1; ++n) {
            T tn, un_1;
            if (n == 0) { tn = T(1); un_1 = T(0); }
            else if (n == 1) { tn = x; un_1 = T(1); }
            else {
                tn = T(2) * x * t_cur - t_prev;
                t_prev = t_cur; t_cur = tn;
                const T un = (n - 1 == 1) ? T(2) * x : T(2) * x * u_prev - u_prev2;
                u_prev2 = u_prev; u_prev = un;
                un_1 = un;
            }
            T td = (n == 0 || zero_d) ? T(0) : T(n) * dxdr * un_1;
            if (out) {
                if (M.fix == 0) { tn += shift * td; td *= damp; }
                else if (M.fix == 2) tn += td * lin;
            }
            if (n >= n0) {
                g[(n - n0) * stride] = tfc * tn;
                h[(n - n0) * stride] = tfc * td + tfd * tn;
            }
        }
    }
}

// FCUT::get_fcut src/Fcut.C:17-72
__device__ __forceinline__ void fcut_eval(const ModelDev& M, double r, double rmax, double& f, double& fd) {
    if (M.fcut == 0) {
        const double irm = 1.0 / rmax;
        double f0 = 1.0 - r * irm;
        f = f0 * f0 * f0;
        fd = f0 * f0 * (-3.0 * irm);
    } else {
        double th = rmax - M.fcut_offset * rmax;
        if (r < th) { f = 1.0; fd = 0.0; }
        else if (r > rmax) { f = 0.0; fd = 0.0; }
        else {
            double a = (r - th) / (rmax - th) * PI_REF + PI_REF / 2.0;
            double ad = PI_REF / (rmax - th);
            f = 0.5 + 0.5 * sin(a);
            fd = 0.5 * cos(a) * ad;
        }
    }
}

__device__ __forceinline__ void edge_members(int NB, int e, int& a, int& b) {
    if (NB == 3) { const int ea[3] = {0, 0, 1}, eb[3] = {1, 2, 2}; a = ea[e]; b = eb[e]; }
    else { const int ea[6] = {0, 0, 0, 1, 1, 2}, eb[6] = {1, 2, 3, 2, 3, 3}; a = ea[e]; b = eb[e]; }
}

__device__ __forceinline__ int member(int4 m, int k) { return k == 0 ? m.x : (k == 1 ? m.y : (k == 2 ? m.z : m.w)); }


// The same basis into registers: g[k] = f T_k(x), h[k] = f T'_k + f' T_k for
// k = 0..O-1 (O a compile-time order, so the arrays stay in registers).  Either
// output may be skipped (WANT_G / WANT_H).
template <int O, bool WANT_G, bool WANT_H, typename R>
__device__ __forceinline__ void basis_regs(const ModelDev& M, double lambda, double xavg, double xdiff, double smin,
                                           double r, double fc, double fd, R* g, R* h) {
    const bool out = r < smin;
    const double rr = out ? smin : r;
    double x, ex = 0.0;
    const double ixd = 1.0 / xdiff;
    if (M.trans == 0) { ex = exp(-rr / lambda); x = (ex - xavg) * ixd; }
    else if (M.trans == 1) { x = (1.0 / rr - xavg) * ixd; }
    else { x = (rr - xavg) * ixd; }
    double dxdr;
    if (M.trans == 0) dxdr = -ex / lambda * ixd;
    else if (M.trans == 1) dxdr = -ixd / (rr * rr);
    else dxdr = ixd;
    dxdr *= M.deriv_const;
    const bool zero_d = out && M.fix == 1;
    double damp = 1.0, shift = 0.0;
    if (out && M.fix == 0) { damp = exp((r - smin) / M.smooth); shift = M.smooth * (damp - 1.0); }
    const double lin = (out && M.fix == 2) ? (r - smin) : 0.0;
    double t_prev = 1.0, t_cur = x, u_prev2 = 0.0, u_prev = 1.0;
#pragma unroll
    for (int n = 0; n < O; ++n) {
        double tn, un_1;
        if (n == 0) { tn = 1.0; un_1 = 0.0; }
        else if (n == 1) { tn = x; un_1 = 1.0; }
        else {
            tn = 2.0 * x * t_cur - t_prev;
            t_prev = t_cur; t_cur = tn;
            const double un = (n - 1 == 1) ? 2.0 * x : 2.0 * x * u_prev - u_prev2;
            u_prev2 = u_prev; u_prev = un;
            un_1 = un;
        }
        double td = (n == 0 || zero_d) ? 0.0 : n * dxdr * un_1;
        if (out) {
            if (M.fix == 0) { tn += shift * td; td *= damp; }
            else if (M.fix == 2) tn += td * lin;
        }
        if (WANT_G) g[n] = R(fc * tn);
        if (WANT_H) h[n] = R(fc * td + fd * tn);
    }
}

// The same recursion with a visitor: v(k, g_k, h_k) for k = 0..count-1 (powers
// n0..n0+count-1), for sums that need no stored basis (the 2-body MD force).
template <typename V>
__device__ __forceinline__ void basis_visit(const ModelDev& M, double lambda, double xavg, double xdiff, double smin,
                                            double r, double fc, double fd, int n0, int count, V& v) {
    const bool out = r < smin;
    const double rr = out ? smin : r;
    double x, ex = 0.0;
    const double ixd = 1.0 / xdiff;
    if (M.trans == 0) { ex = exp(-rr / lambda); x = (ex - xavg) * ixd; }
    else if (M.trans == 1) { x = (1.0 / rr - xavg) * ixd; }
    else { x = (rr - xavg) * ixd; }
    double dxdr;
    if (M.trans == 0) dxdr = -ex / lambda * ixd;
    else if (M.trans == 1) dxdr = -ixd / (rr * rr);
    else dxdr = ixd;
    dxdr *= M.deriv_const;
    const bool zero_d = out && M.fix == 1;
    double damp = 1.0, shift = 0.0;
    if (out && M.fix == 0) { damp = exp((r - smin) / M.smooth); shift = M.smooth * (damp - 1.0); }
    const double lin = (out && M.fix == 2) ? (r - smin) : 0.0;
    double t_prev = 1.0, t_cur = x, u_prev2 = 0.0, u_prev = 1.0;
    const int n1 = n0 + count;
    for (int n = 0; n < n1; ++n) {
        double tn, un_1;
        if (n == 0) { tn = 1.0; un_1 = 0.0; }
        else if (n == 1) { tn = x; un_1 = 1.0; }
        else {
            tn = 2.0 * x * t_cur - t_prev;
            t_prev = t_cur; t_cur = tn;
            const double un = (n - 1 == 1) ? 2.0 * x : 2.0 * x * u_prev - u_prev2;
            u_prev2 = u_prev; u_prev = un;
            un_1 = un;
        }
        double td = (n == 0 || zero_d) ? 0.0 : n * dxdr * un_1;
        if (out) {
            if (M.fix == 0) { tn += shift * td; td *= damp; }
            else if (M.fix == 2) tn += td * lin;
        }
        if (n >= n0) v(n - n0, fc * tn, fc * td + fd * tn);
    }
}

}  // namespace cgd
