/*
 * adjoint2d.cu -- discrete adjoint (reverse mode), tangent-linear model and
 * frozen-dt replay of the 2D MUSCL-Hancock + HLLC step.
 *
 * The differentiated map.  The inputs are the interior primitives W0 =
 * (rho, vx, vy, p); ghost cells are their images under the built-in boundary
 * rules (reflective, transmissive, periodic); U0 is W0 converted to
 * conserved form (src/system.c:884-905).  Step k maps U^k to U^{k+1} with
 * the dt the forward pass chose (dt is frozen: the CFL reduction is not
 * differentiated), W^k = U->W(U^k) for k >= 1 and W^0 = W0.  The output is
 * W^N.  Every limiter, regime and region decision is taken from the primal
 * values of the pass being differentiated, so the derivative is that of the
 * smooth piece the forward pass lies on.
 *
 * Forward pass.  The production step kernel (mh2d_step_kernel) runs the N
 * steps with its own CFL dt; after each step a one-thread kernel logs dt.
 * Every K steps the state (U, W incl. sound speed) and the step-control
 * block are copied aside: a checkpoint.
 *
 * Backward pass.  Segments are processed last to first.  A segment is
 * recomputed from its checkpoint with the production kernel (each step
 * writes its own slab, so all K states stay resident; the recomputed dt is
 * checked against the log and the segment's last state against the next
 * checkpoint, both bit for bit), then swept in reverse:
 *
 *   ad_recon_kernel      face states of step k (x and y, per cell);
 *   ad_flux_vjp_kernel   per face: Fbar from the adjoints of the two cells it
 *                        updates, then the reverse of the HLLC flux;
 *   ad_recon_vjp_kernel  per cell: reverse of the Hancock predictor and the
 *                        limited slopes, split into the cell's own share and
 *                        the shares of its two neighbours per direction;
 *   ad_gather_kernel     per interior cell: gathers the shares (no atomics),
 *                        folds the shares of its ghost images back (the
 *                        reverse of the boundary rule) and applies the
 *                        reverse of U->W, giving Ubar^k (or, at k = 0, the
 *                        reverse of W->U, giving the gradient w.r.t. W0).
 *
 * Tangent-linear model and replay.  The same face-parallel step (recon,
 * flux, update kernels) templated on the number type: Dual runs the
 * tangent-linear model through the very templates the production kernel
 * uses (numerics.cuh), double replays the forward pass from any initial
 * state with the frozen dt and, optionally, sums a hash of every branch
 * decision per step (a branch signature) so that a finite-difference
 * evaluation can tell whether it crossed a kink.
 *
 * The FP64 primal of the replay and of the tangent-linear model is bit-for-
 * bit the production kernel's (same expressions, --fmad=false).
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "adjoint_numerics.cuh"
#include "dual.cuh"
#include "gpu_bridge.h"
#include "gpu_internal.h"

using namespace hydro;

namespace {

constexpr int kThreads = 256;

struct AdGeom {
    int nx, ny, g, tx, ty;      /* tx is the row pitch */
    int bc[4];
};

template <class R>
struct StateP {
    R *W[5];    /* rho, vx, vy, p, sound speed */
    R *U[4];    /* mass, mom_x, mom_y, energy */
};

template <class R>
struct FacesP {
    R *xlo[4], *xhi[4], *ylo[4], *yhi[4];
};

/* Branch codes of one replayed step: planes 0 x reconstruction, 1 y
 * reconstruction, 2 x faces, 3 y faces (one uint16 per padded cell each).
 * rec: record the decisions taken; frc: force these decisions. */
struct BranchP {
    unsigned short *rec[4];
    const unsigned short *frc[4];
};

/* Four device field pointers, passed to kernels by value. */
template <class R>
struct F4 {
    R *p[4];
};

template <class R>
struct FluxP {
    R *fx[4], *fy[4];   /* flux through the high x / y face of each cell */
};

__device__ __forceinline__ bool need_x(const AdGeom &q, int r, int c)
{
    return r >= q.g && r < q.g + q.ny && c >= q.g - 1 && c <= q.g + q.nx;
}

__device__ __forceinline__ bool need_y(const AdGeom &q, int r, int c)
{
    return c >= q.g && c < q.g + q.nx && r >= q.g - 1 && r <= q.g + q.ny;
}

__device__ __forceinline__ bool interior(const AdGeom &q, int r, int c)
{
    return r >= q.g && r < q.g + q.ny && c >= q.g && c < q.g + q.nx;
}

/* Source cell of padded (r, c) under the boundary rules, as fetch_w remaps
 * it for reflective / transmissive / periodic boundaries; neg = 1 flips vx,
 * 2 flips vy. */
__device__ __forceinline__ long long source_cell(const AdGeom &q, int r, int c, int &neg)
{
    int rr = r, cc = c;
    const int g = q.g;
    neg = 0;
    if (c < g) {
        const int k = g - 1 - c, f = q.bc[0];
        if (f == BC_PERIODIC) cc = g + q.nx - 1 - k;
        else { cc = g + k; neg = (f == BC_REFLECTIVE) ? 1 : 0; }
    } else if (c >= g + q.nx) {
        const int k = c - g - q.nx, f = q.bc[1];
        if (f == BC_PERIODIC) cc = g + k;
        else { cc = g + q.nx - 1 - k; neg = (f == BC_REFLECTIVE) ? 1 : 0; }
    } else if (r < g) {
        const int k = g - 1 - r, f = q.bc[2];
        if (f == BC_PERIODIC) rr = g + q.ny - 1 - k;
        else { rr = g + k; neg = (f == BC_REFLECTIVE) ? 2 : 0; }
    } else if (r >= g + q.ny) {
        const int k = r - g - q.ny, f = q.bc[3];
        if (f == BC_PERIODIC) rr = g + k;
        else { rr = g + q.ny - 1 - k; neg = (f == BC_REFLECTIVE) ? 2 : 0; }
    }
    return (long long) rr * q.tx + cc;
}

template <class R>
__device__ __forceinline__ void load_w(const AdGeom &q, R *const *W, int r, int c, R w[4], R &a)
{
    int neg;
    const long long s = source_cell(q, r, c, neg);
#pragma unroll
    for (int k = 0; k < 4; k++) w[k] = W[k][s];
    a = W[4][s];
    if (neg == 1) w[1] = -w[1];
    if (neg == 2) w[2] = -w[2];
}

__device__ __forceinline__ void load_w4(const AdGeom &q, double *const *W, int r, int c, double w[4])
{
    int neg;
    const long long s = source_cell(q, r, c, neg);
#pragma unroll
    for (int k = 0; k < 4; k++) w[k] = W[k][s];
    if (neg == 1) w[1] = -w[1];
    if (neg == 2) w[2] = -w[2];
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ void sig_flush(unsigned long long *sig, unsigned long long h)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0 && h) atomicAdd(sig, h);
}

__device__ __forceinline__ void record(int *err, int code)
{
    atomicCAS(err, 0, code);
}

#define GRID_STRIDE(k, total) \
    for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < (total); \
         k += (long long) gridDim.x * blockDim.x)

/* Row and column of padded index k.  Sessions are created only for grids of
 * fewer than 2^32 padded cells, so 32-bit unsigned arithmetic is exact (a
 * 64-bit integer divide is a long software sequence on the device). */
__device__ __forceinline__ void row_col(const AdGeom &q, long long k, int &r, int &c)
{
    const unsigned kk = (unsigned) k, t = (unsigned) q.tx;
    const unsigned rr = kk / t;
    r = (int) rr;
    c = (int) (kk - rr * t);
}

/* ------------------------------------------------------- forward pieces */

/* Interior: sound speed and U = W->U(W). */
template <class R>
__global__ void ad_init_kernel(const AdGeom q, const GasConst<R> gas, StateP<R> s, R vol)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (!interior(q, r, c)) continue;
        R w[4], U[4];
#pragma unroll
        for (int f = 0; f < 4; f++) w[f] = s.W[f][k];
        s.W[4][k] = sound_speed(gas, w[0], w[3]);
        prim_to_cons_2d(gas, vol, w, U);
#pragma unroll
        for (int f = 0; f < 4; f++) s.U[f][k] = U[f];
    }
}

/* Ghost bands (corners excluded) of fields 0..3 from their source cells. */
__global__ void ad_fill_ghosts_kernel(const AdGeom q, StateP<double> s)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        const bool in_r = r >= q.g && r < q.g + q.ny, in_c = c >= q.g && c < q.g + q.nx;
        if (in_r == in_c) continue;   /* interior or corner */
        double w[4];
        load_w4(q, s.W, r, c, w);
#pragma unroll
        for (int f = 0; f < 4; f++) s.W[f][k] = w[f];
    }
}

/* Face states of every cell a step reads. */
template <class R, int LIM>
__global__ void __launch_bounds__(kThreads) ad_recon_kernel(const AdGeom q, StateP<R> s, FacesP<R> f,
                                                            R dtA_x, R dtA_y, unsigned long long *sig,
                                                            BranchP br)
{
    unsigned long long h = 0;
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        const bool nx_ = need_x(q, r, c), ny_ = need_y(q, r, c);
        if (!nx_ && !ny_) continue;
        R w0[4], a0, t;
        load_w(q, s.W, r, c, w0, a0);
        if (nx_) {
            R wm[4], wp[4], lo[4], hi[4];
            load_w(q, s.W, r, c - 1, wm, t);
            load_w(q, s.W, r, c + 1, wp, t);
            if constexpr (std::is_same<R, double>::value) {
                if (br.frc[0]) recon_cell_forced<LIM>(0, dtA_x, wm, w0, wp, a0, br.frc[0][k], lo, hi);
                else recon_cell<LIM>(0, dtA_x, wm, w0, wp, a0, lo, hi);
                if (sig || br.rec[0]) {
                    const int code = recon_code<LIM>(wm, w0, wp);
                    if (br.rec[0]) br.rec[0][k] = (unsigned short) code;
                    if (sig) h += mix64(((unsigned long long) k << 3) ^ ((unsigned long long) code << 40));
                }
            } else {
                recon_cell<LIM>(0, dtA_x, wm, w0, wp, a0, lo, hi);
            }
#pragma unroll
            for (int e = 0; e < 4; e++) { f.xlo[e][k] = lo[e]; f.xhi[e][k] = hi[e]; }
        }
        if (ny_) {
            R wm[4], wp[4], lo[4], hi[4];
            load_w(q, s.W, r - 1, c, wm, t);
            load_w(q, s.W, r + 1, c, wp, t);
            if constexpr (std::is_same<R, double>::value) {
                if (br.frc[1]) recon_cell_forced<LIM>(1, dtA_y, wm, w0, wp, a0, br.frc[1][k], lo, hi);
                else recon_cell<LIM>(1, dtA_y, wm, w0, wp, a0, lo, hi);
                if (sig || br.rec[1]) {
                    const int code = recon_code<LIM>(wm, w0, wp);
                    if (br.rec[1]) br.rec[1][k] = (unsigned short) code;
                    if (sig) h += mix64(((unsigned long long) k << 3 | 1) ^ ((unsigned long long) code << 40));
                }
            } else {
                recon_cell<LIM>(1, dtA_y, wm, w0, wp, a0, lo, hi);
            }
#pragma unroll
            for (int e = 0; e < 4; e++) { f.ylo[e][k] = lo[e]; f.yhi[e][k] = hi[e]; }
        }
    }
    if constexpr (std::is_same<R, double>::value) {
        if (sig) sig_flush(sig, h);
    }
}

/* HLLC flux through every face a step uses. */
template <class R>
__global__ void __launch_bounds__(kThreads) ad_flux_kernel(const AdGeom q, const GasConst<R> gas, FacesP<R> f,
                                                           FluxP<R> fl, int *err, unsigned long long *sig,
                                                           BranchP br)
{
    unsigned long long h = 0;
    const int g = q.g;
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (r >= g && r < g + q.ny && c >= g - 1 && c <= g + q.nx - 1) {
            R F[4];
            const R L0 = f.xhi[0][k], L1 = f.xhi[1][k], L2 = f.xhi[2][k], L3 = f.xhi[3][k];
            const R R0 = f.xlo[0][k + 1], R1 = f.xlo[1][k + 1], R2 = f.xlo[2][k + 1], R3 = f.xlo[3][k + 1];
            int rc = DEV_OK;
            if constexpr (std::is_same<R, double>::value) {
                if (br.frc[2]) hllc_flux_2d_forced(gas, L0, L1, L2, L3, R0, R1, R2, R3, br.frc[2][k], F);
                else rc = hllc_flux_2d(gas, L0, L1, L2, L3, R0, R1, R2, R3, F);
                if (sig || br.rec[2]) {
                    HllcFwd st;
                    hllc_fwd(gas, L0, L1, L3, R0, R1, R3, st);
                    const int code = hllc_code(gas, st, L0, L1, L3, R0, R1, R3);
                    if (br.rec[2]) br.rec[2][k] = (unsigned short) code;
                    if (sig) h += mix64(((unsigned long long) k << 3 | 2) ^ ((unsigned long long) code << 40));
                }
            } else {
                rc = hllc_flux_2d(gas, L0, L1, L2, L3, R0, R1, R2, R3, F);
            }
            if (rc) record(err, rc);
#pragma unroll
            for (int e = 0; e < 4; e++) fl.fx[e][k] = F[e];
        }
        if (c >= g && c < g + q.nx && r >= g - 1 && r <= g + q.ny - 1) {
            R F[4];
            const long long kn = k + q.tx;
            const R L0 = f.yhi[0][k], L1 = f.yhi[1][k], L2 = f.yhi[2][k], L3 = f.yhi[3][k];
            const R R0 = f.ylo[0][kn], R1 = f.ylo[1][kn], R2 = f.ylo[2][kn], R3 = f.ylo[3][kn];
            int rc = DEV_OK;
            if constexpr (std::is_same<R, double>::value) {
                if (br.frc[3]) hllc_flux_2d_forced(gas, L0, L1, L2, L3, R0, R1, R2, R3, br.frc[3][k], F);
                else rc = hllc_flux_2d(gas, L0, L1, L2, L3, R0, R1, R2, R3, F);
                if (sig || br.rec[3]) {
                    HllcFwd st;
                    hllc_fwd(gas, L0, L1, L3, R0, R1, R3, st);
                    const int code = hllc_code(gas, st, L0, L1, L3, R0, R1, R3);
                    if (br.rec[3]) br.rec[3][k] = (unsigned short) code;
                    if (sig) h += mix64(((unsigned long long) k << 3 | 3) ^ ((unsigned long long) code << 40));
                }
            } else {
                rc = hllc_flux_2d(gas, L0, L1, L2, L3, R0, R1, R2, R3, F);
            }
            if (rc) record(err, rc);
#pragma unroll
            for (int e = 0; e < 4; e++) fl.fy[e][k] = F[e];
        }
    }
    if constexpr (std::is_same<R, double>::value) {
        if (sig) sig_flush(sig, h);
    }
}

/* Conservative update in the production kernel's accumulation order, then
 * U -> W and the sound speed. */
template <class R>
__global__ void __launch_bounds__(kThreads) ad_update_kernel(const AdGeom q, const GasConst<R> gas, StateP<R> in,
                                                             StateP<R> out, FluxP<R> fl, R dtr, R Ax, R Ay, R vol)
{
    const int ymap[4] = { 0, 2, 1, 3 };
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (!interior(q, r, c)) continue;
        R Un[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            R v = in.U[e][k];
            v = v + (fl.fx[e][k - 1] * dtr) * Ax;
            v = v - (fl.fx[e][k] * dtr) * Ax;
            v = v + (fl.fy[ymap[e]][k - q.tx] * dtr) * Ay;
            v = v - (fl.fy[ymap[e]][k] * dtr) * Ay;
            Un[e] = v;
            out.U[e][k] = v;
        }
        R w[4];
        cons_to_prim_2d(gas, vol, Un[0], Un[1], Un[2], Un[3], w);
#pragma unroll
        for (int e = 0; e < 4; e++) out.W[e][k] = w[e];
        out.W[4][k] = sound_speed(gas, w[0], w[3]);
    }
}

/* (value, tangent) double arrays -> Dual interior. */
__global__ void ad_pack_dual_kernel(const AdGeom q, F4<double> w, F4<double> dw, StateP<Dual> s)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (!interior(q, r, c)) continue;
#pragma unroll
        for (int f = 0; f < 4; f++) s.W[f][k] = Dual(w.p[f][k], dw.p[f][k]);
    }
}

/* Dual interior -> value and tangent arrays (ghost entries zero). */
__global__ void ad_unpack_dual_kernel(const AdGeom q, StateP<Dual> s, F4<double> w, F4<double> dw)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        const bool in = interior(q, r, c);
#pragma unroll
        for (int f = 0; f < 4; f++) {
            const Dual x = in ? s.W[f][k] : Dual(0.0, 0.0);
            w.p[f][k] = x.v;
            dw.p[f][k] = x.d;
        }
    }
}

/* Interior of 4 fields into an output with zero ghost entries. */
__global__ void ad_copy_interior_kernel(const AdGeom q, F4<double> src, F4<double> dst)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        const bool in = interior(q, r, c);
#pragma unroll
        for (int f = 0; f < 4; f++) dst.p[f][k] = in ? src.p[f][k] : 0.0;
    }
}

/* ------------------------------------------------------ stepping control */

__global__ void ad_log_dt_kernel(const HydroStepControl *ctrl, double *dt_log, long long n)
{
    dt_log[n] = ctrl->dt;
}

__global__ void ad_check_dt_kernel(const HydroStepControl *ctrl, const double *dt_log, long long n,
                                   unsigned long long *mismatch)
{
    if (ctrl->dt != dt_log[n] || ctrl->error_code != 0) atomicAdd(mismatch, 1ull);
}

/* Interior cells whose recomputed U differs (bitwise) from the stored one. */
__global__ void ad_compare_kernel(const AdGeom q, StateP<double> a, StateP<double> b, unsigned long long *mismatch)
{
    unsigned long long n = 0;
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (!interior(q, r, c)) continue;
        bool diff = false;
#pragma unroll
        for (int f = 0; f < 4; f++) {
            const double x = a.U[f][k], y = b.U[f][k];
            diff |= __double_as_longlong(x) != __double_as_longlong(y);
        }
        n += diff ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(mismatch, n);
}

/* ---------------------------------------------------------- reverse sweep */

/* Ubar^N = reverse of U->W applied to the seed dJ/dW^N. */
__global__ void ad_seed_kernel(const AdGeom q, const GasConst<double> gas, double vol, StateP<double> s,
                               F4<double> seed, F4<double> Ub)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (!interior(q, r, c)) continue;
        const double wb[4] = { seed.p[0][k], seed.p[1][k], seed.p[2][k], seed.p[3][k] };
        double ub[4] = { 0, 0, 0, 0 };
        cons_to_prim_2d_vjp(gas, vol, s.U[0][k], s.U[1][k], s.U[2][k], wb, ub);
#pragma unroll
        for (int f = 0; f < 4; f++) Ub.p[f][k] = ub[f];
    }
}

/* Per face: Fbar = dt * area * (Ubar of the cell above - Ubar of the cell
 * below) (ghost Ubar is zero: ghost U is not state), then the reverse of the
 * HLLC flux into the adjoints of the two face states. */
__global__ void __launch_bounds__(kThreads, 2) ad_flux_vjp_kernel(const AdGeom q, const GasConst<double> gas,
                                                               FacesP<double> f, FacesP<double> fb,
                                                               F4<double> Ub, double cx, double cy, int *err)
{
    const int g = q.g;
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (r >= g && r < g + q.ny && c >= g - 1 && c <= g + q.nx - 1) {
            double L[4], Rs[4], Fb[4], Lb[4], Rb[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                L[e] = f.xhi[e][k];
                Rs[e] = f.xlo[e][k + 1];
                Fb[e] = cx * (Ub.p[e][k + 1] - Ub.p[e][k]);
            }
            const int rc = hllc_vjp(gas, L, Rs, Fb, Lb, Rb, nullptr);
            if (rc) record(err, rc);
#pragma unroll
            for (int e = 0; e < 4; e++) { fb.xhi[e][k] = Lb[e]; fb.xlo[e][k + 1] = Rb[e]; }
        }
        if (c >= g && c < g + q.nx && r >= g - 1 && r <= g + q.ny - 1) {
            const long long kn = k + q.tx;
            double L[4], Rs[4], Fb[4], Lb[4], Rb[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                L[e] = f.yhi[e][k];
                Rs[e] = f.ylo[e][kn];
            }
            /* y flux components are (mass, mom_y, mom_x, energy) */
            Fb[0] = cy * (Ub.p[0][kn] - Ub.p[0][k]);
            Fb[1] = cy * (Ub.p[2][kn] - Ub.p[2][k]);
            Fb[2] = cy * (Ub.p[1][kn] - Ub.p[1][k]);
            Fb[3] = cy * (Ub.p[3][kn] - Ub.p[3][k]);
            const int rc = hllc_vjp(gas, L, Rs, Fb, Lb, Rb, nullptr);
            if (rc) record(err, rc);
#pragma unroll
            for (int e = 0; e < 4; e++) { fb.yhi[e][k] = Lb[e]; fb.ylo[e][kn] = Rb[e]; }
        }
    }
}

/* Reverse HLLC of one face from the tape the recomputation wrote (face
 * states, the HLLC guess with its factors, and the wave-speed factors and
 * S*), so neither the reconstruction, the guesses nor the wave speeds are
 * evaluated again.  dir 0: the x face above cell k, dir 1: the y face. */
__device__ __forceinline__ void flux_vjp_tape_face(const AdGeom &q, const GasConst<double> &gas,
                                                   const double *tape, long long plane, FacesP<double> &fb,
                                                   const F4<double> &Ub, double cx, double cy, int *err,
                                                   long long k, int dir)
{
    const double *T = tape + (long long) (dir * MH2D_TAPE_FIELDS) * plane + k;
    const long long kn = dir == 0 ? k + 1 : k + q.tx;
    double L[4], Rs[4], Fb[4], Lb[4], Rb[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
        L[e] = T[(TAPE_L + e) * plane];
        Rs[e] = T[(TAPE_R + e) * plane];
    }
    if (dir == 0) {
#pragma unroll
        for (int e = 0; e < 4; e++) Fb[e] = cx * (Ub.p[e][kn] - Ub.p[e][k]);
    } else {
        /* y flux components are (mass, mom_y, mom_x, energy) */
        Fb[0] = cy * (Ub.p[0][kn] - Ub.p[0][k]);
        Fb[1] = cy * (Ub.p[2][kn] - Ub.p[2][k]);
        Fb[2] = cy * (Ub.p[1][kn] - Ub.p[1][k]);
        Fb[3] = cy * (Ub.p[3][kn] - Ub.p[3][k]);
    }
    HllcFwd st;
    const int rc = hllc_fwd_from_tape(gas, L[0], L[1], L[3], Rs[0], Rs[1], Rs[3], T[TAPE_AL * plane],
                                      T[TAPE_AR * plane], T[TAPE_PG * plane], (int) T[TAPE_REG * plane],
                                      T[TAPE_QL * plane], T[TAPE_QR * plane], T[TAPE_SS * plane], st);
    if (rc) {
        record(err, rc);
#pragma unroll
        for (int e = 0; e < 4; e++) { Lb[e] = 0.0; Rb[e] = 0.0; }
    } else {
        hllc_vjp_core(gas, L, Rs, st, true, T[TAPE_Z0 * plane], T[TAPE_Z1 * plane], Fb, Lb, Rb);
    }
    if (dir == 0) {
#pragma unroll
        for (int e = 0; e < 4; e++) { fb.xhi[e][k] = Lb[e]; fb.xlo[e][kn] = Rb[e]; }
    } else {
#pragma unroll
        for (int e = 0; e < 4; e++) { fb.yhi[e][k] = Lb[e]; fb.ylo[e][kn] = Rb[e]; }
    }
}

/* Whether cell k owns an x face (dir 0) or a y face (dir 1) of the sweep. */
__device__ __forceinline__ bool owns_face(const AdGeom &q, int r, int c, int dir)
{
    const int g = q.g;
    return dir == 0 ? (r >= g && r < g + q.ny && c >= g - 1 && c <= g + q.nx - 1)
                    : (c >= g && c < g + q.nx && r >= g - 1 && r <= g + q.ny - 1);
}

/* Faces of one step binned by their taped guess regime (PREG_*: vacuum,
 * PVRS, two-rarefaction, two-shock), so that the reverse HLLC runs warps of
 * one regime (the regimes' reverse code differs; mixed warps serialise
 * over it).  A face is 2k + dir; bins[b * cap + i], counts[b].  Appends are
 * aggregated per warp and regime. */
__global__ void ad_face_bins_kernel(const AdGeom q, const double *tape, long long plane, unsigned *bins,
                                    unsigned *counts, long long cap)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
#pragma unroll
        for (int dir = 0; dir < 2; dir++) {
            if (!owns_face(q, r, c, dir)) continue;
            const int b = (int) tape[(long long) (dir * MH2D_TAPE_FIELDS + TAPE_REG) * plane + k] & 3;
            const unsigned mask = __activemask();
            const unsigned peers = __match_any_sync(mask, b);
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(peers) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(&counts[b], (unsigned) __popc(peers));
            base = __shfl_sync(peers, base, leader);
            const unsigned pos = base + (unsigned) __popc(peers & ((1u << lane) - 1u));
            bins[(long long) b * cap + pos] = (unsigned) (2 * k + dir);
        }
    }
}

/* The reverse HLLC over the binned faces: PVRS, two-rarefaction, two-shock,
 * then vacuum faces. */
__global__ void __launch_bounds__(kThreads, 2) ad_flux_vjp_bins_kernel(const AdGeom q, const GasConst<double> gas,
                                                                     const double *tape, long long plane,
                                                                     FacesP<double> fb, F4<double> Ub, double cx,
                                                                     double cy, int *err, const unsigned *bins,
                                                                     const unsigned *counts, long long cap)
{
    const unsigned n1 = counts[PREG_PVRS], n2 = counts[PREG_TRRS], n3 = counts[PREG_TSRS];
    const unsigned n0 = counts[PREG_VACUUM];
    const long long total = (long long) n0 + n1 + n2 + n3;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < total;
         i += (long long) gridDim.x * blockDim.x) {
        int b;
        long long j = i;
        if (j < n1) b = PREG_PVRS;
        else if ((j -= n1) < n2) b = PREG_TRRS;
        else if ((j -= n2) < n3) b = PREG_TSRS;
        else { j -= n3; b = PREG_VACUUM; }
        const unsigned id = bins[(long long) b * cap + j];
        flux_vjp_tape_face(q, gas, tape, plane, fb, Ub, cx, cy, err, (long long) (id >> 1), (int) (id & 1u));
    }
}

/* Shares of the reverse reconstruction (storage order rho, vx, vy, p). */
struct SharesP {
    double *own[4];
    double *Ax[4], *Bx[4], *Ay[4], *By[4];
};

template <int LIM>
__global__ void __launch_bounds__(kThreads) ad_recon_vjp_kernel(const AdGeom q, const GasConst<double> gas,
                                                                StateP<double> s, FacesP<double> fb,
                                                                SharesP sh, double dtA_x, double dtA_y)
{
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        const bool nx_ = need_x(q, r, c), ny_ = need_y(q, r, c);
        if (!nx_ && !ny_) continue;
        double w0[4], a0, o[4] = { 0, 0, 0, 0 };
        load_w(q, s.W, r, c, w0, a0);
        const double inv_rho = rv(w0[0]), inv_p = rv(w0[3]);
        if (nx_) {
            double wm[4], wp[4], lob[4], hib[4], ox[4], A[4], B[4];
            load_w4(q, s.W, r, c - 1, wm);
            load_w4(q, s.W, r, c + 1, wp);
#pragma unroll
            for (int e = 0; e < 4; e++) { lob[e] = fb.xlo[e][k]; hib[e] = fb.xhi[e][k]; }
            recon_cell_vjp<LIM>(0, dtA_x, wm, w0, wp, a0, inv_rho, inv_p, lob, hib, ox, A, B);
#pragma unroll
            for (int e = 0; e < 4; e++) { o[e] += ox[e]; sh.Ax[e][k] = A[e]; sh.Bx[e][k] = B[e]; }
        }
        if (ny_) {
            double wm[4], wp[4], lob[4], hib[4], oy[4], A[4], B[4];
            load_w4(q, s.W, r - 1, c, wm);
            load_w4(q, s.W, r + 1, c, wp);
#pragma unroll
            for (int e = 0; e < 4; e++) { lob[e] = fb.ylo[e][k]; hib[e] = fb.yhi[e][k]; }
            recon_cell_vjp<LIM>(1, dtA_y, wm, w0, wp, a0, inv_rho, inv_p, lob, hib, oy, A, B);
#pragma unroll
            for (int e = 0; e < 4; e++) { o[e] += oy[e]; sh.Ay[e][k] = A[e]; sh.By[e][k] = B[e]; }
        }
#pragma unroll
        for (int e = 0; e < 4; e++) sh.own[e][k] = o[e];
    }
}

/* Adjoint reaching padded cell (r, c) as read by the step: its own share
 * plus the shares its four neighbours' slopes send it. */
__device__ __forceinline__ void gather_cell(const AdGeom &q, const SharesP &sh, int r, int c, double o[4])
{
    const long long k = (long long) r * q.tx + c;
    const bool self = need_x(q, r, c) || need_y(q, r, c);
    const bool xp = need_x(q, r, c + 1), xm = need_x(q, r, c - 1);
    const bool yp = need_y(q, r + 1, c), ym = need_y(q, r - 1, c);
#pragma unroll
    for (int e = 0; e < 4; e++) {
        double v = self ? sh.own[e][k] : 0.0;
        if (xp) v -= sh.Ax[e][k + 1];
        if (xm) v += sh.Bx[e][k - 1];
        if (yp) v -= sh.Ay[e][k + q.tx];
        if (ym) v += sh.By[e][k - q.tx];
        o[e] = v;
    }
}

/* Per interior cell: gather, fold in the ghost images (reverse of the
 * boundary rule), then Ubar^k = Ubar^{k+1} + reverse(U->W), or at k = 0 the
 * gradient w.r.t. W0 = Wbar + reverse(W->U)(Ubar^1). */
__global__ void __launch_bounds__(kThreads) ad_gather_kernel(const AdGeom q, const GasConst<double> gas, double vol,
                                                             SharesP sh, StateP<double> s, F4<double> Ub,
                                                             int first, F4<double> grad)
{
    const int g = q.g;
    GRID_STRIDE(k, (long long) q.tx * q.ty) {
        int r, c;
        row_col(q, k, r, c);
        if (!interior(q, r, c)) continue;
        double wb[4];
        gather_cell(q, sh, r, c, wb);
        /* ghost images: depth 0 and 1 on each side */
#pragma unroll
        for (int side = 0; side < 4; side++) {
            const int f = q.bc[side];
#pragma unroll
            for (int d = 0; d < 2; d++) {
                int gr = r, gc = c, src;
                if (side == 0) { gc = g - 1 - d; src = (f == BC_PERIODIC) ? g + q.nx - 1 - d : g + d; if (src != c) continue; }
                else if (side == 1) { gc = g + q.nx + d; src = (f == BC_PERIODIC) ? g + d : g + q.nx - 1 - d; if (src != c) continue; }
                else if (side == 2) { gr = g - 1 - d; src = (f == BC_PERIODIC) ? g + q.ny - 1 - d : g + d; if (src != r) continue; }
                else { gr = g + q.ny + d; src = (f == BC_PERIODIC) ? g + d : g + q.ny - 1 - d; if (src != r) continue; }
                double o[4];
                gather_cell(q, sh, gr, gc, o);
                if (f == BC_REFLECTIVE) {
                    if (side < 2) o[1] = -o[1];
                    else o[2] = -o[2];
                }
#pragma unroll
                for (int e = 0; e < 4; e++) wb[e] += o[e];
            }
        }
        if (!first) {
            double ub[4] = { Ub.p[0][k], Ub.p[1][k], Ub.p[2][k], Ub.p[3][k] };
            cons_to_prim_2d_vjp(gas, vol, s.U[0][k], s.U[1][k], s.U[2][k], wb, ub);
#pragma unroll
            for (int e = 0; e < 4; e++) Ub.p[e][k] = ub[e];
        } else {
            const double w[4] = { s.W[0][k], s.W[1][k], s.W[2][k], s.W[3][k] };
            const double ub[4] = { Ub.p[0][k], Ub.p[1][k], Ub.p[2][k], Ub.p[3][k] };
            prim_to_cons_2d_vjp(gas, vol, w, ub, wb);
#pragma unroll
            for (int e = 0; e < 4; e++) grad.p[e][k] = wb[e];
        }
    }
}

int grid_for(long long n)
{
    long long b = (n + kThreads - 1) / kThreads;
    if (b > 152 * 16) b = 152 * 16;
    return (int) (b < 1 ? 1 : b);
}

}  // namespace

/* ================================================================ runtime */

struct HydroAdj2D {
    HydroGrid2D grid{};
    HydroGpuOptions opt{};
    HydroStepParams sp{};
    AdGeom geom{};
    int device = 0;
    long long nsteps = 0;
    int K = 1;
    int n_ckpt = 0;                    /* checkpoints at steps 0, K, 2K, ... < nsteps */
    size_t ncell = 0, fbytes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {};
    std::vector<void *> allocs;
    /* state sets of 9 fields: U[4], W[5] */
    std::vector<StateP<double>> ckpt;  /* n_ckpt */
    std::vector<StateP<double>> seg;   /* K slabs for steps k0+1 .. k0+K */
    StateP<double> fwd[2]{};
    StateP<double> fin{};               /* points at fwd[nsteps & 1] after the forward pass */
    HydroStepControl *ctrl_d = nullptr;
    HydroStepControl *ckpt_ctrl_d = nullptr;
    HydroStepControl *ctrl_h = nullptr;
    double *dt_log_d = nullptr;
    std::vector<double> dt_h;
    unsigned long long *counters_d = nullptr;  /* [0] recompute mismatches, [1] dt mismatches */
    unsigned long long *sig_d = nullptr;       /* branch signature per replayed step */
    unsigned short *codes_d = nullptr;         /* forward branch codes, nsteps x 4 planes (on demand) */
    bool have_codes = false;
    int *err_d = nullptr;
    Mh2dArgs<double> pargs{};
    /* face-parallel stepper (double): replay and the reverse sweep's faces */
    StateP<double> gen[2]{};
    FacesP<double> faces{};
    FluxP<double> flux{};
    /* reverse sweep */
    FacesP<double> faces_b{};
    SharesP shares{};
    double *Ub[4] = {};
    double *stage[8] = {};             /* host transfer staging (8 fields) */
    /* tangent-linear model (allocated on first use) */
    bool have_tlm = false;
    StateP<Dual> tgen[2]{};
    FacesP<Dual> tfaces{};
    FluxP<Dual> tflux{};
    bool forward_done = false;
    /* tape of a segment (K steps x 2 x MH2D_TAPE_FIELDS fields), written by the
     * recomputation and read by the reverse sweep */
    bool use_tape = true;
    double *tape_d = nullptr;
    /* faces of a step binned by regime for the reverse HLLC (4 x 2 ncell) */
    unsigned *bins_d = nullptr;
    unsigned *bin_counts_d = nullptr;
    /* statistics */
    double forward_ms = 0, recompute_ms = 0, vjp_ms = 0, tangent_ms = 0, replay_ms = 0;
    long long launches = 0;
    long long device_bytes = 0;
    unsigned long long recompute_mismatches = 0;
};

namespace {

void set_err(HydroRunOutcome *oc, cudaError_t e, const char *what)
{
    if (!oc) return;
    oc->kind = HYDRO_RUN_CUDA_ERROR;
    oc->code = (int) e;
    snprintf(oc->message, sizeof oc->message, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                          \
    do {                                        \
        cudaError_t e_ = (call);                \
        if (e_ != cudaSuccess) {                \
            set_err(oc, e_, what);              \
            return -1;                          \
        }                                       \
    } while (0)

int dalloc(HydroAdj2D *a, size_t bytes, void **p, HydroRunOutcome *oc)
{
    CK(cudaMalloc(p, bytes), "cudaMalloc(adjoint)");
    a->allocs.push_back(*p);
    a->device_bytes += (long long) bytes;
    CK(cudaMemsetAsync(*p, 0, bytes, a->stream), "cudaMemset(adjoint)");
    return 0;
}

/* n fields of `elem` bytes each, zeroed. */
template <class R>
int fields(HydroAdj2D *a, int n, R **out, HydroRunOutcome *oc)
{
    void *p;
    if (dalloc(a, (size_t) n * a->ncell * sizeof(R), &p, oc)) return -1;
    for (int i = 0; i < n; i++) out[i] = static_cast<R *>(p) + (size_t) i * a->ncell;
    return 0;
}

template <class R>
int state_fields(HydroAdj2D *a, StateP<R> &s, HydroRunOutcome *oc)
{
    R *f[9];
    if (fields<R>(a, 9, f, oc)) return -1;
    for (int i = 0; i < 4; i++) s.U[i] = f[i];
    for (int i = 0; i < 5; i++) s.W[i] = f[4 + i];
    return 0;
}

template <class R>
int faces_fields(HydroAdj2D *a, FacesP<R> &fc, HydroRunOutcome *oc)
{
    R *f[16];
    if (fields<R>(a, 16, f, oc)) return -1;
    for (int i = 0; i < 4; i++) {
        fc.xlo[i] = f[i];
        fc.xhi[i] = f[4 + i];
        fc.ylo[i] = f[8 + i];
        fc.yhi[i] = f[12 + i];
    }
    return 0;
}

template <class R>
int flux_fields(HydroAdj2D *a, FluxP<R> &fl, HydroRunOutcome *oc)
{
    R *f[8];
    if (fields<R>(a, 8, f, oc)) return -1;
    for (int i = 0; i < 4; i++) { fl.fx[i] = f[i]; fl.fy[i] = f[4 + i]; }
    return 0;
}

int copy_state(HydroAdj2D *a, const StateP<double> &src, const StateP<double> &dst, HydroRunOutcome *oc)
{
    for (int i = 0; i < 4; i++)
        CK(cudaMemcpyAsync(dst.U[i], src.U[i], a->fbytes, cudaMemcpyDeviceToDevice, a->stream), "D2D state");
    for (int i = 0; i < 5; i++)
        CK(cudaMemcpyAsync(dst.W[i], src.W[i], a->fbytes, cudaMemcpyDeviceToDevice, a->stream), "D2D state");
    return 0;
}

/* One production step n from `in` to `out`. */
int prod_step(HydroAdj2D *a, long long n, const StateP<double> &in, const StateP<double> &out,
              double *tape, HydroRunOutcome *oc)
{
    Mh2dArgs<double> args = a->pargs;
    const int b = (int) (n & 1);
    for (int i = 0; i < 4; i++) { args.U[b][i] = in.U[i]; args.U[b ^ 1][i] = out.U[i]; }
    for (int i = 0; i < 5; i++) { args.W[b][i] = in.W[i]; args.W[b ^ 1][i] = out.W[i]; }
    if (tape) {
        args.tape = tape;
        args.tape_plane = (long long) a->ncell;
        CK(mh2d_launch_step_tape<double>(args, a->grid.limiter, a->stream), "step kernel (tape)");
    } else {
        CK(mh2d_launch_step<double>(args, a->grid.limiter, a->stream), "step kernel");
    }
    a->launches++;
    return 0;
}

int check_err(HydroAdj2D *a, HydroRunOutcome *oc)
{
    int err = 0;
    CK(cudaMemcpyAsync(&err, a->err_d, sizeof(int), cudaMemcpyDeviceToHost, a->stream), "D2H error");
    CK(cudaStreamSynchronize(a->stream), "adjoint");
    if (err) {
        oc->kind = HYDRO_RUN_DEVICE_ERROR;
        oc->code = err;
        snprintf(oc->message, sizeof oc->message, "Device error %d in the adjoint step kernels.", err);
        return -1;
    }
    return 0;
}

template <class R>
int launch_recon(HydroAdj2D *a, StateP<R> s, FacesP<R> f, double dt, unsigned long long *sig, BranchP br,
                 HydroRunOutcome *oc)
{
    const R dtA_x = R(dt * a->grid.area_x / a->grid.vol);
    const R dtA_y = R(dt * a->grid.area_y / a->grid.vol);
    const int nb = grid_for((long long) a->ncell);
    switch (a->grid.limiter) {
    case LIM_MINMOD:
        ad_recon_kernel<R, LIM_MINMOD><<<nb, kThreads, 0, a->stream>>>(a->geom, s, f, dtA_x, dtA_y, sig, br);
        break;
    case LIM_VAN_LEER:
        ad_recon_kernel<R, LIM_VAN_LEER><<<nb, kThreads, 0, a->stream>>>(a->geom, s, f, dtA_x, dtA_y, sig, br);
        break;
    default:
        ad_recon_kernel<R, LIM_MC><<<nb, kThreads, 0, a->stream>>>(a->geom, s, f, dtA_x, dtA_y, sig, br);
        break;
    }
    CK(cudaGetLastError(), "recon kernel");
    a->launches++;
    return 0;
}

/* One face-parallel step n of the replay (double) or tangent-linear (Dual) model. */
template <class R>
int gen_step(HydroAdj2D *a, long long n, StateP<R> in, StateP<R> out, FacesP<R> f, FluxP<R> fl,
             unsigned long long *sig, BranchP br, HydroRunOutcome *oc)
{
    const double dt = a->dt_h[(size_t) n];
    const int nb = grid_for((long long) a->ncell);
    if (launch_recon<R>(a, in, f, dt, sig, br, oc)) return -1;
    const GasConst<R> gas = make_gas_const<R>(a->grid.gamma, a->grid.tol);
    ad_flux_kernel<R><<<nb, kThreads, 0, a->stream>>>(a->geom, gas, f, fl, a->err_d, sig, br);
    CK(cudaGetLastError(), "flux kernel");
    ad_update_kernel<R><<<nb, kThreads, 0, a->stream>>>(a->geom, gas, in, out, fl, R(dt), R(a->grid.area_x),
                                                        R(a->grid.area_y), R(a->grid.vol));
    CK(cudaGetLastError(), "update kernel");
    a->launches += 2;
    return 0;
}

F4<double> f4(double *const p[4])
{
    F4<double> r;
    for (int i = 0; i < 4; i++) r.p[i] = p[i];
    return r;
}

int upload4(HydroAdj2D *a, double *const host[4], double *const dev[4], HydroRunOutcome *oc)
{
    for (int i = 0; i < 4; i++)
        CK(cudaMemcpyAsync(dev[i], host[i], a->fbytes, cudaMemcpyHostToDevice, a->stream), "H2D");
    return 0;
}

int download4(HydroAdj2D *a, double *const dev[4], double *const host[4], HydroRunOutcome *oc)
{
    for (int i = 0; i < 4; i++)
        CK(cudaMemcpyAsync(host[i], dev[i], a->fbytes, cudaMemcpyDeviceToHost, a->stream), "D2H");
    return 0;
}

int ensure_tlm(HydroAdj2D *a, HydroRunOutcome *oc)
{
    if (a->have_tlm) return 0;
    if (state_fields<Dual>(a, a->tgen[0], oc) || state_fields<Dual>(a, a->tgen[1], oc) ||
        faces_fields<Dual>(a, a->tfaces, oc) || flux_fields<Dual>(a, a->tflux, oc))
        return -1;
    a->have_tlm = true;
    return 0;
}

float elapsed(HydroAdj2D *a, int e0, int e1)
{
    float ms = 0;
    cudaEventElapsedTime(&ms, a->ev[e0], a->ev[e1]);
    return ms;
}

}  // namespace

extern "C" int hydro_adj2d_create(const HydroGrid2D *grid, const HydroGpuOptions *opt, const HydroStepParams *sp,
                                  int64 num_steps, int checkpoint_every, double *const W0[4],
                                  HydroAdj2D **out, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    *out = nullptr;
    if (grid->integrator != INTEGRATOR_MUSCL_HANCOCK_2D) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "The adjoint differentiates muscl_hancock_2d only.");
        return -1;
    }
    for (int s = 0; s < 4; s++) {
        if (grid->bc[s] != BC_REFLECTIVE && grid->bc[s] != BC_TRANSMISSIVE && grid->bc[s] != BC_PERIODIC) {
            oc->kind = HYDRO_RUN_UNSUPPORTED;
            snprintf(oc->message, sizeof oc->message,
                     "The adjoint needs reflective, transmissive or periodic boundaries.");
            return -1;
        }
    }
    if (grid->g < 2 || grid->nx < 2 || grid->ny < 2 || num_steps < 1 || checkpoint_every < 1 ||
        opt->precision != HYDRO_GPU_PRECISION_FP64) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message,
                 "The adjoint needs G >= 2, at least 2 x 2 cells, num_steps >= 1, checkpoint_every >= 1 and FP64.");
        return -1;
    }
    if ((long long) (grid->nx + 2 * grid->g) * (grid->ny + 2 * grid->g) >= (1ll << 32)) {
        oc->kind = HYDRO_RUN_UNSUPPORTED;
        snprintf(oc->message, sizeof oc->message, "The adjoint needs fewer than 2^32 padded cells.");
        return -1;
    }
    HydroAdj2D *a = new (std::nothrow) HydroAdj2D();
    if (!a) {
        oc->kind = HYDRO_RUN_CUDA_ERROR;
        snprintf(oc->message, sizeof oc->message, "Host allocation failed.");
        return -1;
    }
    *out = a;
    a->grid = *grid;
    a->opt = *opt;
    a->sp = *sp;
    a->sp.is_storing = 0;
    a->device = opt->device;
    a->nsteps = num_steps;
    a->K = (int) (checkpoint_every < num_steps ? checkpoint_every : num_steps);
    a->n_ckpt = (int) ((num_steps + a->K - 1) / a->K);
    const int tx = grid->nx + 2 * grid->g, ty = grid->ny + 2 * grid->g;
    a->ncell = (size_t) tx * ty;

    a->fbytes = a->ncell * sizeof(double);
    a->geom.nx = grid->nx;
    a->geom.ny = grid->ny;
    a->geom.g = grid->g;
    a->geom.tx = tx;
    a->geom.ty = ty;
    for (int s = 0; s < 4; s++) a->geom.bc[s] = grid->bc[s];

    CK(cudaSetDevice(a->device), "cudaSetDevice");
    CK(cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    for (auto &e : a->ev) CK(cudaEventCreate(&e), "cudaEventCreate");
    a->ckpt.resize((size_t) a->n_ckpt);
    a->seg.resize((size_t) a->K);
    for (auto &s : a->ckpt)
        if (state_fields<double>(a, s, oc)) return -1;
    for (auto &s : a->seg)
        if (state_fields<double>(a, s, oc)) return -1;
    for (auto &s : a->fwd)
        if (state_fields<double>(a, s, oc)) return -1;
    for (auto &s : a->gen)
        if (state_fields<double>(a, s, oc)) return -1;
    if (faces_fields<double>(a, a->faces, oc) || flux_fields<double>(a, a->flux, oc) ||
        faces_fields<double>(a, a->faces_b, oc))
        return -1;
    {
        double *f[20];
        if (fields<double>(a, 20, f, oc)) return -1;
        for (int i = 0; i < 4; i++) {
            a->shares.own[i] = f[i];
            a->shares.Ax[i] = f[4 + i];
            a->shares.Bx[i] = f[8 + i];
            a->shares.Ay[i] = f[12 + i];
            a->shares.By[i] = f[16 + i];
        }
    }
    if (fields<double>(a, 4, a->Ub, oc) || fields<double>(a, 8, a->stage, oc)) return -1;
    void *p;
    if (dalloc(a, sizeof(HydroStepControl), &p, oc)) return -1;
    a->ctrl_d = static_cast<HydroStepControl *>(p);
    if (dalloc(a, (size_t) a->n_ckpt * sizeof(HydroStepControl), &p, oc)) return -1;
    a->ckpt_ctrl_d = static_cast<HydroStepControl *>(p);
    if (dalloc(a, (size_t) num_steps * sizeof(double), &p, oc)) return -1;
    a->dt_log_d = static_cast<double *>(p);
    if (dalloc(a, 4 * sizeof(unsigned long long), &p, oc)) return -1;
    a->counters_d = static_cast<unsigned long long *>(p);
    if (dalloc(a, (size_t) num_steps * sizeof(unsigned long long), &p, oc)) return -1;
    a->sig_d = static_cast<unsigned long long *>(p);
    if (dalloc(a, sizeof(int), &p, oc)) return -1;
    a->err_d = static_cast<int *>(p);
    CK(cudaMallocHost(&a->ctrl_h, sizeof(HydroStepControl)), "cudaMallocHost(control)");

    /* production-kernel arguments (buffers are set per step) */
    Mh2dArgs<double> &pa = a->pargs;
    pa.ctrl = a->ctrl_d;
    pa.sp = a->sp;
    pa.gas = make_gas_const<double>(grid->gamma, grid->tol);
    pa.nx = grid->nx;
    pa.ny = grid->ny;
    pa.g = grid->g;
    pa.pitch = tx;
    pa.strip_w = mh2d_threads<double>() - 2;
    for (int s = 0; s < 4; s++) pa.bc[s] = grid->bc[s];
    pa.dx = grid->dx;
    pa.dy = grid->dy;
    pa.area_x = grid->area_x;
    pa.area_y = grid->area_y;
    pa.vol = grid->vol;
    pa.first_order = 0;
    pa.grid_ctas = mh2d_resident_ctas<double>(grid->limiter, 0, a->device);
    pa.chunk_h = opt->chunk_rows > 0 ? opt->chunk_rows
                                     : mh2d_default_chunk(pa.nx, pa.ny, pa.strip_w, pa.grid_ctas);

    /* initial state: interior W0, ghosts from the boundary rules, U0 = W->U(W0) */
    StateP<double> s0 = a->ckpt[0];
    if (upload4(a, W0, s0.W, oc)) return -1;
    const int nb = grid_for((long long) a->ncell);
    ad_fill_ghosts_kernel<<<nb, kThreads, 0, a->stream>>>(a->geom, s0);
    CK(cudaGetLastError(), "ghost kernel");
    ad_init_kernel<double><<<nb, kThreads, 0, a->stream>>>(a->geom, pa.gas, s0, grid->vol);
    CK(cudaGetLastError(), "init kernel");
    a->launches += 2;
    CK(cudaStreamSynchronize(a->stream), "adjoint create");
    return 0;
}

extern "C" int hydro_adj2d_forward(HydroAdj2D *a, double *const W[4], double *const U[4], HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    CK(cudaSetDevice(a->device), "cudaSetDevice");
    HydroStepControl *c = a->ctrl_h;
    memset(c, 0, sizeof *c);
    c->tf = 1e300;
    c->max_steps = a->nsteps;
    c->active = 1;
    const unsigned long long ninf = ordered_bits(-INFINITY);
    for (int k = 0; k < 3; k++) c->smax[k][0] = c->smax[k][1] = ninf;
    CK(cudaEventRecord(a->ev[0], a->stream), "cudaEventRecord");
    CK(cudaMemcpyAsync(a->ctrl_d, c, sizeof *c, cudaMemcpyHostToDevice, a->stream), "H2D control");
    /* sound speed everywhere and the first CFL maxima, from checkpoint 0 */
    Mh2dArgs<double> args = a->pargs;
    for (int i = 0; i < 5; i++) args.W[0][i] = a->ckpt[0].W[i];
    CK(mh2d_launch_prepare<double>(args, a->stream), "prepare kernel");
    a->launches++;
    CK(cudaMemcpyAsync(&a->ckpt_ctrl_d[0], a->ctrl_d, sizeof *c, cudaMemcpyDeviceToDevice, a->stream), "D2D control");
    const StateP<double> *in = &a->ckpt[0];
    for (long long n = 0; n < a->nsteps; n++) {
        const StateP<double> &o = a->fwd[(n + 1) & 1];
        if (prod_step(a, n, *in, o, nullptr, oc)) return -1;
        ad_log_dt_kernel<<<1, 1, 0, a->stream>>>(a->ctrl_d, a->dt_log_d, n);
        CK(cudaGetLastError(), "dt log kernel");
        a->launches++;
        const long long nn = n + 1;
        if (nn < a->nsteps && nn % a->K == 0) {
            const int ci = (int) (nn / a->K);
            if (copy_state(a, o, a->ckpt[(size_t) ci], oc)) return -1;
            CK(cudaMemcpyAsync(&a->ckpt_ctrl_d[ci], a->ctrl_d, sizeof *c, cudaMemcpyDeviceToDevice, a->stream),
               "D2D control");
        }
        in = &o;
    }
    a->fin = *in;
    CK(cudaEventRecord(a->ev[1], a->stream), "cudaEventRecord");
    CK(cudaMemcpyAsync(c, a->ctrl_d, sizeof *c, cudaMemcpyDeviceToHost, a->stream), "D2H control");
    CK(cudaStreamSynchronize(a->stream), "adjoint forward");
    a->forward_ms = elapsed(a, 0, 1);
    oc->num_steps = c->num_steps;
    oc->t = c->t;
    oc->dt = c->dt;
    if (c->error_code != 0) {
        oc->kind = HYDRO_RUN_DEVICE_ERROR;
        oc->code = c->error_code;
        oc->where = c->error_cell;
        snprintf(oc->message, sizeof oc->message, "Device error %d in the forward pass.", c->error_code);
        return -1;
    }
    if (c->num_steps != a->nsteps) {
        oc->kind = HYDRO_RUN_DEVICE_ERROR;
        snprintf(oc->message, sizeof oc->message, "The forward pass stopped after %lld of %lld steps.",
                 (long long) c->num_steps, (long long) a->nsteps);
        return -1;
    }
    a->dt_h.resize((size_t) a->nsteps);
    CK(cudaMemcpy(a->dt_h.data(), a->dt_log_d, (size_t) a->nsteps * sizeof(double), cudaMemcpyDeviceToHost),
       "D2H dt log");
    a->forward_done = true;
    if (W) {
        double *st[4] = { a->stage[0], a->stage[1], a->stage[2], a->stage[3] };
        ad_copy_interior_kernel<<<grid_for((long long) a->ncell), kThreads, 0, a->stream>>>(a->geom, f4(a->fin.W), f4(st));
        CK(cudaGetLastError(), "copy kernel");
        a->launches++;
        if (download4(a, st, W, oc)) return -1;
    }
    if (U) {
        double *st[4] = { a->stage[4], a->stage[5], a->stage[6], a->stage[7] };
        ad_copy_interior_kernel<<<grid_for((long long) a->ncell), kThreads, 0, a->stream>>>(a->geom, f4(a->fin.U), f4(st));
        CK(cudaGetLastError(), "copy kernel");
        a->launches++;
        if (download4(a, st, U, oc)) return -1;
    }
    CK(cudaStreamSynchronize(a->stream), "adjoint forward");
    return 0;
}

static int need_forward(HydroAdj2D *a, HydroRunOutcome *oc)
{
    if (a->forward_done) return 0;
    oc->kind = HYDRO_RUN_UNSUPPORTED;
    snprintf(oc->message, sizeof oc->message, "Run the forward pass first.");
    return -1;
}

extern "C" int hydro_adj2d_backward(HydroAdj2D *a, double *const seed[4], double *const grad[4],
                                    HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    if (need_forward(a, oc)) return -1;
    CK(cudaSetDevice(a->device), "cudaSetDevice");
    const AdGeom q = a->geom;
    const int nb = grid_for((long long) a->ncell);
    const GasConst<double> gas = make_gas_const<double>(a->grid.gamma, a->grid.tol);
    const double vol = a->grid.vol;
    CK(cudaMemsetAsync(a->err_d, 0, sizeof(int), a->stream), "memset");
    CK(cudaMemsetAsync(a->counters_d, 0, 4 * sizeof(unsigned long long), a->stream), "memset");
    double *sd[4] = { a->stage[0], a->stage[1], a->stage[2], a->stage[3] };
    if (upload4(a, seed, sd, oc)) return -1;
    ad_seed_kernel<<<nb, kThreads, 0, a->stream>>>(q, gas, vol, a->fin, f4(sd), f4(a->Ub));
    CK(cudaGetLastError(), "seed kernel");
    a->launches++;
    a->recompute_ms = 0;
    a->vjp_ms = 0;
    double *tape_base = nullptr;
    if (a->use_tape) {
        if (!a->tape_d) {
            void *p;
            if (dalloc(a, (size_t) a->K * 2 * MH2D_TAPE_FIELDS * a->ncell * sizeof(double), &p, oc)) return -1;
            a->tape_d = static_cast<double *>(p);
            if (dalloc(a, (size_t) 4 * 2 * a->ncell * sizeof(unsigned), &p, oc)) return -1;
            a->bins_d = static_cast<unsigned *>(p);
            if (dalloc(a, 4 * sizeof(unsigned), &p, oc)) return -1;
            a->bin_counts_d = static_cast<unsigned *>(p);
        }
        tape_base = a->tape_d;
    }
    for (int s = a->n_ckpt - 1; s >= 0; s--) {
        const long long k0 = (long long) s * a->K;
        const long long k1 = (k0 + a->K < a->nsteps) ? k0 + a->K : a->nsteps;
        auto slab = [&](long long k) -> const StateP<double> & {
            return (k == k0) ? a->ckpt[(size_t) s] : a->seg[(size_t) (k - k0 - 1)];
        };
        /* ---- recompute the segment with the production kernel ---- */
        CK(cudaEventRecord(a->ev[0], a->stream), "cudaEventRecord");
        CK(cudaMemcpyAsync(a->ctrl_d, &a->ckpt_ctrl_d[s], sizeof(HydroStepControl), cudaMemcpyDeviceToDevice,
                           a->stream), "D2D control");
        auto tape_of = [&](long long k) -> double * {
            return tape_base ? tape_base + (size_t) (k - k0) * 2 * MH2D_TAPE_FIELDS * a->ncell : nullptr;
        };
        for (long long n = k0; n < k1; n++) {
            if (prod_step(a, n, slab(n), slab(n + 1), tape_of(n), oc)) return -1;
            ad_check_dt_kernel<<<1, 1, 0, a->stream>>>(a->ctrl_d, a->dt_log_d, n, a->counters_d + 1);
            CK(cudaGetLastError(), "dt check kernel");
            a->launches++;
        }
        const StateP<double> &ref = (k1 == a->nsteps) ? a->fin : a->ckpt[(size_t) (s + 1)];
        ad_compare_kernel<<<nb, kThreads, 0, a->stream>>>(q, slab(k1), ref, a->counters_d);
        CK(cudaGetLastError(), "compare kernel");
        a->launches++;
        CK(cudaEventRecord(a->ev[1], a->stream), "cudaEventRecord");
        /* ---- reverse sweep over the segment ---- */
        for (long long k = k1 - 1; k >= k0; k--) {
            const StateP<double> &st = slab(k);
            const double dt = a->dt_h[(size_t) k];
            if (tape_base) {
                const long long cap = 2 * (long long) a->ncell;
                CK(cudaMemsetAsync(a->bin_counts_d, 0, 4 * sizeof(unsigned), a->stream), "cudaMemset(bins)");
                ad_face_bins_kernel<<<nb, kThreads, 0, a->stream>>>(q, tape_of(k), (long long) a->ncell, a->bins_d,
                                                                    a->bin_counts_d, cap);
                CK(cudaGetLastError(), "face bins kernel");
                ad_flux_vjp_bins_kernel<<<grid_for(cap), kThreads, 0, a->stream>>>(
                    q, gas, tape_of(k), (long long) a->ncell, a->faces_b, f4(a->Ub), dt * a->grid.area_x,
                    dt * a->grid.area_y, a->err_d, a->bins_d, a->bin_counts_d, cap);
                CK(cudaGetLastError(), "flux vjp kernel");
                a->launches++;
            } else {
                if (launch_recon<double>(a, st, a->faces, dt, nullptr, BranchP{}, oc)) return -1;
                ad_flux_vjp_kernel<<<nb, kThreads, 0, a->stream>>>(q, gas, a->faces, a->faces_b, f4(a->Ub),
                                                                   dt * a->grid.area_x, dt * a->grid.area_y,
                                                                   a->err_d);
                CK(cudaGetLastError(), "flux vjp kernel");
            }
            const double dtA_x = dt * a->grid.area_x / vol, dtA_y = dt * a->grid.area_y / vol;
            switch (a->grid.limiter) {
            case LIM_MINMOD:
                ad_recon_vjp_kernel<LIM_MINMOD><<<nb, kThreads, 0, a->stream>>>(q, gas, st, a->faces_b, a->shares, dtA_x, dtA_y);
                break;
            case LIM_VAN_LEER:
                ad_recon_vjp_kernel<LIM_VAN_LEER><<<nb, kThreads, 0, a->stream>>>(q, gas, st, a->faces_b, a->shares, dtA_x, dtA_y);
                break;
            default:
                ad_recon_vjp_kernel<LIM_MC><<<nb, kThreads, 0, a->stream>>>(q, gas, st, a->faces_b, a->shares, dtA_x, dtA_y);
                break;
            }
            CK(cudaGetLastError(), "recon vjp kernel");
            double *gd[4] = { a->stage[4], a->stage[5], a->stage[6], a->stage[7] };
            ad_gather_kernel<<<nb, kThreads, 0, a->stream>>>(q, gas, vol, a->shares, st, f4(a->Ub), k == 0 ? 1 : 0, f4(gd));
            CK(cudaGetLastError(), "gather kernel");
            a->launches += 3;
        }
        CK(cudaEventRecord(a->ev[2], a->stream), "cudaEventRecord");
        CK(cudaEventSynchronize(a->ev[2]), "adjoint segment");
        a->recompute_ms += elapsed(a, 0, 1);
        a->vjp_ms += elapsed(a, 1, 2);
    }
    unsigned long long cnt[2] = { 0, 0 };
    CK(cudaMemcpyAsync(cnt, a->counters_d, sizeof cnt, cudaMemcpyDeviceToHost, a->stream), "D2H counters");
    if (check_err(a, oc)) return -1;
    a->recompute_mismatches = cnt[0] + cnt[1];
    double *gd[4] = { a->stage[4], a->stage[5], a->stage[6], a->stage[7] };
    /* ghost entries of the gradient are zero: clear them in the staging copy */
    double *go[4] = { a->stage[0], a->stage[1], a->stage[2], a->stage[3] };
    ad_copy_interior_kernel<<<nb, kThreads, 0, a->stream>>>(q, f4(gd), f4(go));
    CK(cudaGetLastError(), "copy kernel");
    a->launches++;
    if (download4(a, go, grad, oc)) return -1;
    CK(cudaStreamSynchronize(a->stream), "adjoint backward");
    return 0;
}

extern "C" int hydro_adj2d_tangent(HydroAdj2D *a, double *const w0[4], double *const dw0[4],
                                   double *const wN[4], double *const dwN[4], HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    if (need_forward(a, oc)) return -1;
    CK(cudaSetDevice(a->device), "cudaSetDevice");
    if (ensure_tlm(a, oc)) return -1;
    const int nb = grid_for((long long) a->ncell);
    CK(cudaMemsetAsync(a->err_d, 0, sizeof(int), a->stream), "memset");
    double *sw[4] = { a->stage[0], a->stage[1], a->stage[2], a->stage[3] };
    double *sd[4] = { a->stage[4], a->stage[5], a->stage[6], a->stage[7] };
    if (w0) {
        if (upload4(a, w0, sw, oc)) return -1;
    } else {
        for (int i = 0; i < 4; i++)
            CK(cudaMemcpyAsync(sw[i], a->ckpt[0].W[i], a->fbytes, cudaMemcpyDeviceToDevice, a->stream), "D2D");
    }
    if (upload4(a, dw0, sd, oc)) return -1;
    CK(cudaEventRecord(a->ev[0], a->stream), "cudaEventRecord");
    ad_pack_dual_kernel<<<nb, kThreads, 0, a->stream>>>(a->geom, f4(sw), f4(sd), a->tgen[0]);
    CK(cudaGetLastError(), "pack kernel");
    const GasConst<Dual> gas = make_gas_const<Dual>(a->grid.gamma, a->grid.tol);
    ad_init_kernel<Dual><<<nb, kThreads, 0, a->stream>>>(a->geom, gas, a->tgen[0], Dual(a->grid.vol));
    CK(cudaGetLastError(), "init kernel");
    a->launches += 2;
    for (long long n = 0; n < a->nsteps; n++) {
        if (gen_step<Dual>(a, n, a->tgen[n & 1], a->tgen[(n + 1) & 1], a->tfaces, a->tflux, nullptr, BranchP{}, oc))
            return -1;
    }
    ad_unpack_dual_kernel<<<nb, kThreads, 0, a->stream>>>(a->geom, a->tgen[a->nsteps & 1], f4(sw), f4(sd));
    CK(cudaGetLastError(), "unpack kernel");
    a->launches++;
    CK(cudaEventRecord(a->ev[1], a->stream), "cudaEventRecord");
    if (check_err(a, oc)) return -1;
    a->tangent_ms = elapsed(a, 0, 1);
    if (wN && download4(a, sw, wN, oc)) return -1;
    if (download4(a, sd, dwN, oc)) return -1;
    CK(cudaStreamSynchronize(a->stream), "adjoint tangent");
    return 0;
}

/* Replay of the forward pass from w0 with the logged dt.  mode 0: branches
 * decided by the replay itself (optionally hashed into per-step
 * signatures); mode 1: the forward pass's branch decisions forced (recorded
 * once, by a replay from W0, into nsteps x 4 code planes). */
static int replay_run(HydroAdj2D *a, const StateP<double> &init, int mode, unsigned long long *sig,
                      HydroRunOutcome *oc)
{
    const GasConst<double> gas = make_gas_const<double>(a->grid.gamma, a->grid.tol);
    const int nb = grid_for((long long) a->ncell);
    for (int i = 0; i < 4; i++)
        CK(cudaMemcpyAsync(a->gen[0].W[i], init.W[i], a->fbytes, cudaMemcpyDeviceToDevice, a->stream), "D2D");
    ad_init_kernel<double><<<nb, kThreads, 0, a->stream>>>(a->geom, gas, a->gen[0], a->grid.vol);
    CK(cudaGetLastError(), "init kernel");
    a->launches++;
    for (long long n = 0; n < a->nsteps; n++) {
        BranchP br{};
        for (int pl = 0; pl < 4; pl++) {
            unsigned short *plane = a->codes_d ? a->codes_d + ((size_t) n * 4 + pl) * a->ncell : nullptr;
            if (mode == 1) br.frc[pl] = plane;
            if (mode == 2) br.rec[pl] = plane;
        }
        if (gen_step<double>(a, n, a->gen[n & 1], a->gen[(n + 1) & 1], a->faces, a->flux,
                             sig ? sig + n : nullptr, br, oc))
            return -1;
    }
    return 0;
}

static int ensure_codes(HydroAdj2D *a, HydroRunOutcome *oc)
{
    if (a->have_codes) return 0;
    if (!a->codes_d) {
        void *p;
        if (dalloc(a, (size_t) a->nsteps * 4 * a->ncell * sizeof(unsigned short), &p, oc)) return -1;
        a->codes_d = static_cast<unsigned short *>(p);
    }
    if (replay_run(a, a->ckpt[0], 2, nullptr, oc)) return -1;
    if (check_err(a, oc)) return -1;
    a->have_codes = true;
    return 0;
}

extern "C" int hydro_adj2d_replay(HydroAdj2D *a, double *const w0[4], double *const wN[4],
                                  unsigned long long *signatures, int frozen, HydroRunOutcome *oc)
{
    memset(oc, 0, sizeof *oc);
    if (need_forward(a, oc)) return -1;
    CK(cudaSetDevice(a->device), "cudaSetDevice");
    const int nb = grid_for((long long) a->ncell);
    CK(cudaMemsetAsync(a->err_d, 0, sizeof(int), a->stream), "memset");
    if (frozen && ensure_codes(a, oc)) return -1;
    unsigned long long *sig = (signatures && !frozen) ? a->sig_d : nullptr;
    if (sig) CK(cudaMemsetAsync(sig, 0, (size_t) a->nsteps * sizeof(unsigned long long), a->stream), "memset");
    /* the initial W goes to the second replay state first (the run copies it in) */
    StateP<double> init = a->gen[1];
    if (upload4(a, w0, init.W, oc)) return -1;
    CK(cudaEventRecord(a->ev[0], a->stream), "cudaEventRecord");
    if (replay_run(a, init, frozen ? 1 : 0, sig, oc)) return -1;
    double *sw[4] = { a->stage[0], a->stage[1], a->stage[2], a->stage[3] };
    ad_copy_interior_kernel<<<nb, kThreads, 0, a->stream>>>(a->geom, f4(a->gen[a->nsteps & 1].W), f4(sw));
    CK(cudaGetLastError(), "copy kernel");
    a->launches++;
    CK(cudaEventRecord(a->ev[1], a->stream), "cudaEventRecord");
    if (check_err(a, oc)) return -1;
    a->replay_ms = elapsed(a, 0, 1);
    if (download4(a, sw, wN, oc)) return -1;
    if (sig)
        CK(cudaMemcpyAsync(signatures, sig, (size_t) a->nsteps * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           a->stream), "D2H signatures");
    CK(cudaStreamSynchronize(a->stream), "adjoint replay");
    return 0;
}

extern "C" void hydro_adj2d_set_tape(HydroAdj2D *a, int enabled)
{
    a->use_tape = enabled != 0;
}

extern "C" int hydro_adj2d_dt(const HydroAdj2D *a, double *dt)
{
    if (!a->forward_done) return -1;
    memcpy(dt, a->dt_h.data(), a->dt_h.size() * sizeof(double));
    return 0;
}

extern "C" void hydro_adj2d_stats(const HydroAdj2D *a, HydroGpuAdjointStats *st)
{
    memset(st, 0, sizeof *st);
    st->forward_ms = a->forward_ms;
    st->recompute_ms = a->recompute_ms;
    st->vjp_ms = a->vjp_ms;
    st->tangent_ms = a->tangent_ms;
    st->replay_ms = a->replay_ms;
    st->steps = a->nsteps;
    st->checkpoint_every = a->K;
    st->checkpoints = a->n_ckpt;
    st->recompute_mismatches = (int64) a->recompute_mismatches;
    st->kernel_launches = a->launches;
    st->device_bytes = a->device_bytes;
    st->interior_cells = (int64) a->grid.nx * a->grid.ny;
}

extern "C" void hydro_adj2d_destroy(HydroAdj2D *a)
{
    if (!a) return;
    cudaSetDevice(a->device);
    if (a->stream) cudaStreamSynchronize(a->stream);
    for (void *p : a->allocs) cudaFree(p);
    if (a->ctrl_h) cudaFreeHost(a->ctrl_h);
    for (auto &e : a->ev)
        if (e) cudaEventDestroy(e);
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a;
}
