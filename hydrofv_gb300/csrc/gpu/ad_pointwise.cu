/*
 * ad_pointwise.cu -- host builds of the pointwise derivative code: the
 * tangent-linear (Dual through numerics.cuh) and reverse-mode
 * (adjoint_numerics.cuh) forms of the HLLC 2D flux and of one cell's
 * MUSCL-Hancock reconstruction.  They let the derivative pieces be checked
 * against each other and against finite differences without a GPU; the
 * adjoint kernels compile the same templates for the device.
 */
#include "adjoint_numerics.cuh"
#include "dual.cuh"
#include "hydro_gpu.h"

using namespace hydro;

extern "C" int hydro_ad_hllc_jvp(double gamma, double tol, const double L[4], const double R[4],
                                 const double dL[4], const double dR[4], double F[4], double dF[4])
{
    const GasConst<Dual> c = make_gas_const<Dual>(gamma, tol);
    Dual Fd[4];
    const int rc = hllc_flux_2d(c, Dual(L[0], dL[0]), Dual(L[1], dL[1]), Dual(L[2], dL[2]), Dual(L[3], dL[3]),
                                Dual(R[0], dR[0]), Dual(R[1], dR[1]), Dual(R[2], dR[2]), Dual(R[3], dR[3]), Fd);
    for (int q = 0; q < 4; q++) { F[q] = Fd[q].v; dF[q] = Fd[q].d; }
    return rc;
}

extern "C" int hydro_ad_hllc_vjp(double gamma, double tol, const double L[4], const double R[4],
                                 const double Fb[4], double Lb[4], double Rb[4], int *branch_code)
{
    const GasConst<double> c = make_gas_const<double>(gamma, tol);
    return hllc_vjp(c, L, R, Fb, Lb, Rb, branch_code);
}

template <int LIM>
static void recon_jvp(int dir, double gamma, double dtA, const double wm[4], const double w0[4],
                      const double wp[4], const double dwm[4], const double dw0[4], const double dwp[4],
                      double lo[4], double hi[4], double dlo[4], double dhi[4])
{
    const GasConst<Dual> c = make_gas_const<Dual>(gamma, 0.0);
    Dual m[4], z[4], p[4], l[4], h[4];
    for (int q = 0; q < 4; q++) {
        m[q] = Dual(wm[q], dwm[q]);
        z[q] = Dual(w0[q], dw0[q]);
        p[q] = Dual(wp[q], dwp[q]);
    }
    const Dual a0 = sound_speed(c, z[0], z[3]);
    recon_cell<LIM>(dir, Dual(dtA), m, z, p, a0, l, h);
    for (int q = 0; q < 4; q++) { lo[q] = l[q].v; dlo[q] = l[q].d; hi[q] = h[q].v; dhi[q] = h[q].d; }
}

extern "C" void hydro_ad_recon_jvp(int limiter, int dir, double gamma, double dtA, const double wm[4],
                                   const double w0[4], const double wp[4], const double dwm[4],
                                   const double dw0[4], const double dwp[4], double lo[4], double hi[4],
                                   double dlo[4], double dhi[4])
{
    if (limiter == LIM_MINMOD) recon_jvp<LIM_MINMOD>(dir, gamma, dtA, wm, w0, wp, dwm, dw0, dwp, lo, hi, dlo, dhi);
    else if (limiter == LIM_VAN_LEER) recon_jvp<LIM_VAN_LEER>(dir, gamma, dtA, wm, w0, wp, dwm, dw0, dwp, lo, hi, dlo, dhi);
    else recon_jvp<LIM_MC>(dir, gamma, dtA, wm, w0, wp, dwm, dw0, dwp, lo, hi, dlo, dhi);
}

extern "C" void hydro_ad_recon_vjp(int limiter, int dir, double gamma, double dtA, const double wm[4],
                                   const double w0[4], const double wp[4], const double lob[4],
                                   const double hib[4], double wmb[4], double w0b[4], double wpb[4])
{
    const GasConst<double> c = make_gas_const<double>(gamma, 0.0);
    double own[4], A[4], B[4];
    const double a0 = sound_speed(c, w0[0], w0[3]), ir = 1.0 / w0[0], ip = 1.0 / w0[3];
    if (limiter == LIM_MINMOD) recon_cell_vjp<LIM_MINMOD>(dir, dtA, wm, w0, wp, a0, ir, ip, lob, hib, own, A, B);
    else if (limiter == LIM_VAN_LEER) recon_cell_vjp<LIM_VAN_LEER>(dir, dtA, wm, w0, wp, a0, ir, ip, lob, hib, own, A, B);
    else recon_cell_vjp<LIM_MC>(dir, dtA, wm, w0, wp, a0, ir, ip, lob, hib, own, A, B);
    for (int q = 0; q < 4; q++) {
        w0b[q] = own[q];
        wmb[q] = -A[q];
        wpb[q] = B[q];
    }
}

extern "C" void hydro_ad_hllc_forced(double gamma, double tol, const double L[4], const double R[4], int code,
                                     double F[4])
{
    const GasConst<double> c = make_gas_const<double>(gamma, tol);
    hllc_flux_2d_forced(c, L[0], L[1], L[2], L[3], R[0], R[1], R[2], R[3], code, F);
}

extern "C" void hydro_ad_recon_forced(int limiter, int dir, double gamma, double dtA, const double wm[4],
                                      const double w0[4], const double wp[4], int code, double lo[4],
                                      double hi[4], int *natural_code)
{
    const GasConst<double> c = make_gas_const<double>(gamma, 0.0);
    const double a0 = sound_speed(c, w0[0], w0[3]);
    if (limiter == LIM_MINMOD) {
        recon_cell_forced<LIM_MINMOD>(dir, dtA, wm, w0, wp, a0, code, lo, hi);
        *natural_code = recon_code<LIM_MINMOD>(wm, w0, wp);
    } else if (limiter == LIM_VAN_LEER) {
        recon_cell_forced<LIM_VAN_LEER>(dir, dtA, wm, w0, wp, a0, code, lo, hi);
        *natural_code = recon_code<LIM_VAN_LEER>(wm, w0, wp);
    } else {
        recon_cell_forced<LIM_MC>(dir, dtA, wm, w0, wp, a0, code, lo, hi);
        *natural_code = recon_code<LIM_MC>(wm, w0, wp);
    }
}
