/*
 * mh2d_kernel.cuh -- fused, unsplit MUSCL-Hancock + HLLC step for 2D
 * Cartesian grids (one kernel launch per time step).
 *
 * Replaces, for one step, src/integrator_muscl_hancock.c:530-1144 (dt, the
 * x and y sweeps, the conservative update), src/system.c:763-802 (U -> W),
 * src/boundary.c:513-777 (built-in ghost cells) and src/utils.c:55-95 (the
 * next step's CFL maxima).
 *
 * Work decomposition ("strip marching"): a CTA of NT threads owns a strip of
 * NT-2 interior columns and a chunk of rows, and marches up the rows.  Thread
 * t is bound to column c0-1+t; it reconstructs that column's cell in x for
 * the current row (slots 0..sw+1 include one halo cell per side) and solves
 * the x face between slot t and t+1, so every x face in the strip is solved
 * once.  In y each interior thread carries its column upwards: the cell
 * above is reconstructed once, the face between them is solved once, and the
 * top-face state and face flux roll over to the next row.  Only the two halo
 * columns per strip and one extra row of y work per chunk are redundant.
 *
 * W rows live in a 3-row shared-memory ring (5 fields: rho, u, v, p and the
 * sound speed a, which the previous step's epilogue already computed), so a
 * cell's W is read from HBM once per CTA.  Ghost cells are never stored:
 * they are produced on load by index remapping (mirror, mirror with a sign
 * flip, or periodic wrap), which yields exactly the values the reference's
 * boundary routine copies.  For "none" boundaries the ghost primitives are
 * converted from the ghost conserved values, as the reference's all-cell
 * conversion does.
 *
 * The update is a gather in the reference's accumulation order
 * U += F_{i-1/2}; U -= F_{i+1/2}; U += G_{j-1/2}; U -= G_{j+1/2}, each term
 * (flux*dt)*area (formed once per face), so no atomics and no scatter
 * races.  The first ghost layer receives its one-sided update too (the
 * reference updates it and the "none" boundary reads it back).  The epilogue converts the new U to W, stores both
 * and folds a+|u|, a+|v| into CTA maxima that become the next step's dt.
 *
 * Both the state and W are double-buffered (step n reads buffer n&1 and
 * writes the other), so CTAs never read a halo another CTA has already
 * overwritten.  Step 0 reads the caller's primitives raw (ghosts included),
 * matching the reference, whose first step uses the W arrays as handed in.
 */
#ifndef HYDRO_GPU_MH2D_KERNEL_CUH
#define HYDRO_GPU_MH2D_KERNEL_CUH

#include <cuda_runtime.h>
#include <math_constants.h>

#include "numerics.cuh"
#include "step_control.h"

/* Threads per 2D step CTA (a strip of threads - 2 interior columns) and the
 * CTAs per SM each state precision is compiled for (launch bounds).  FP64:
 * 4 CTAs of 128 threads (128 registers); FP32: 7 CTAs of 128 (72
 * registers).  Measured with the one-pass FP32 face solve (2048^2 shear
 * layer / 8192^2 point blast / 256-grid ensemble, G cell-updates/s): 8 CTAs
 * 15.05 / 27.5 / 20.1, 7 CTAs 15.19 / 28.6 / 21.35, 6 CTAs 15.7 / 27.7 /
 * 20.4. */
#ifndef MH2D_THREADS_FP64
#define MH2D_THREADS_FP64 128
#endif
#ifndef MH2D_CTAS_FP64
#define MH2D_CTAS_FP64 4
#endif
#ifndef MH2D_THREADS_FP32
#define MH2D_THREADS_FP32 128
#endif
#ifndef MH2D_CTAS_FP32
#define MH2D_CTAS_FP32 7
#endif

namespace hydro {

template <class R>
constexpr int mh2d_threads() { return sizeof(R) == 8 ? MH2D_THREADS_FP64 : MH2D_THREADS_FP32; }

/* The same, for host code that holds the precision as a flag. */
inline int mh2d_threads_for(bool fp32) { return fp32 ? MH2D_THREADS_FP32 : MH2D_THREADS_FP64; }

template <class R>
struct Mh2dArgs {
    R *U[2][4];              /* [buffer][mass, mom_x, mom_y, energy] */
    R *W[2][5];              /* [buffer][rho, u, v, p, a] */
    HydroStepControl *ctrl;
    HydroStepParams sp;
    GasConst<R> gas;
    int nx, ny, g, pitch;
    int strip_w;             /* interior columns per strip (NT - 2) */
    int chunk_h;             /* rows per work item */
    int tail_h, tail_rows;   /* the last tail_rows rows go in items of tail_h rows, queued
                              * after the others (0: every item has chunk_h rows) */
    int bc[4];               /* x_min, x_max, y_min, y_max */
    double dx, dy;           /* System.dx_, dy_ (for dt) */
    double area_x, area_y, vol;
    int first_order;         /* 1: Godunov first order (face states = cell states) */
    int grid_ctas;           /* persistent CTAs per step launch (0: one per work item) */
    double gravity;          /* System.gravity (kernels built with GRAV only) */
    R *tape;                 /* adjoint tape of this step (kernels built with TAPE only) */
    long long tape_plane;    /* elements per tape field (padded cells) */
};

/* Work items of one step: (strip, row chunk) pairs, chunk-major, so the
 * queue hands out all strips of a chunk before the next chunk.  Rows
 * [0, ny - tail_rows) come in chunks of chunk_h rows, the rest in chunks of
 * tail_h rows: the short items come last and fill the persistent CTAs' last
 * round. */
template <class R>
__host__ __device__ inline int mh2d_n_items(const Mh2dArgs<R> &a)
{
    const int strips = (a.nx + a.strip_w - 1) / a.strip_w;
    const int big = a.ny - a.tail_rows;
    int chunks = (big + a.chunk_h - 1) / a.chunk_h;
    if (a.tail_rows > 0) chunks += (a.tail_rows + a.tail_h - 1) / a.tail_h;
    return strips * chunks;
}

/* Strip and padded row range [r0, r1) of work item `item`. */
template <class R>
__host__ __device__ inline void mh2d_item_rows(const Mh2dArgs<R> &a, int item, int &strip, int &r0, int &r1)
{
    const int strips = (a.nx + a.strip_w - 1) / a.strip_w;
    strip = item % strips;
    const int k = item / strips;
    const int big = a.ny - a.tail_rows;
    const int nbig = (big + a.chunk_h - 1) / a.chunk_h;
    int lo, hi;
    if (k < nbig) {
        lo = k * a.chunk_h;
        hi = (lo + a.chunk_h < big) ? lo + a.chunk_h : big;
    } else {
        lo = big + (k - nbig) * a.tail_h;
        hi = (lo + a.tail_h < a.ny) ? lo + a.tail_h : a.ny;
    }
    r0 = a.g + lo;
    r1 = a.g + hi;
}

/*
 * Adjoint tape of one step (written by the TAPE build of the step kernel,
 * read by the reverse sweep).  Per face, at the padded index of its left
 * (x faces) or lower (y faces) cell, MH2D_TAPE_FIELDS fields per direction
 * (x fields first, then y): the face states (4 + 4, normal velocity in
 * slot 1), both sound speeds, the star-pressure guess before the floor, the
 * guess's factors (p^((g-1)/2g) of each side for the two-rarefaction guess,
 * g_K of each side for the two-shock guess), the regime, and the wave-speed
 * factors q_L, q_R and S* of the finish (zero for vacuum faces).
 */
#define MH2D_TAPE_FIELDS 17
enum : int {
    TAPE_L = 0, TAPE_R = 4, TAPE_AL = 8, TAPE_AR = 9, TAPE_PG = 10, TAPE_Z0 = 11, TAPE_Z1 = 12,
    TAPE_REG = 13, TAPE_QL = 14, TAPE_QR = 15, TAPE_SS = 16,
};

/* Where solve_faces writes the tape of a batch: faces [0, nxf) are x faces
 * of row row_x with left cells c0-1+f; the rest are y faces between row_y
 * and row_y+1 in columns c0+(f-nxf). */
template <class R>
struct TapeCtx {
    R *tape;
    long long plane;
    int pitch, nxf, row_x, row_y, c0;
    __device__ __forceinline__ R *field(int f, int q) const
    {
        const bool x = f < nxf;
        const long long idx = x ? (long long) row_x * pitch + c0 - 1 + f
                                : (long long) row_y * pitch + c0 + (f - nxf);
        return tape + ((x ? 0 : MH2D_TAPE_FIELDS) + q) * plane + idx;
    }
};

/* Where W at padded (r, c) comes from: the stored cell (rr, cc), with the
 * sign of u (neg = 1) or v (neg = 2) flipped, or (cons) converted from the
 * stored U of (rr, cc).  Ghost cells map to their source; ghost cells of
 * custom (host callback) sides are read as stored: the host wrote them
 * after the previous step. */
template <class R>
__device__ __forceinline__ void w_source(const Mh2dArgs<R> &a, bool raw, int r, int c, int &rr, int &cc,
                                         int &neg, bool &cons)
{
    rr = r;
    cc = c;
    neg = 0;
    cons = false;
    if (!raw) {
        const int g = a.g, nx = a.nx, ny = a.ny;
        int f = 0, k = 0;
        if (c < g) {
            f = a.bc[0]; k = g - 1 - c;
            if (f == BC_NONE) cons = true;
            else if (f == BC_PERIODIC) cc = g + nx - 1 - k;
            else if (f != BC_CUSTOM) { cc = g + k; neg = (f == BC_REFLECTIVE) ? 1 : 0; }
        } else if (c >= g + nx) {
            f = a.bc[1]; k = c - g - nx;
            if (f == BC_NONE) cons = true;
            else if (f == BC_PERIODIC) cc = g + k;
            else if (f != BC_CUSTOM) { cc = g + nx - 1 - k; neg = (f == BC_REFLECTIVE) ? 1 : 0; }
        } else if (r < g) {
            f = a.bc[2]; k = g - 1 - r;
            if (f == BC_NONE) cons = true;
            else if (f == BC_PERIODIC) rr = g + ny - 1 - k;
            else if (f != BC_CUSTOM) { rr = g + k; neg = (f == BC_REFLECTIVE) ? 2 : 0; }
        } else if (r >= g + ny) {
            f = a.bc[3]; k = r - g - ny;
            if (f == BC_NONE) cons = true;
            else if (f == BC_PERIODIC) rr = g + k;
            else if (f != BC_CUSTOM) { rr = g + ny - 1 - k; neg = (f == BC_REFLECTIVE) ? 2 : 0; }
        }
    }
}

/* Load W at padded (r, c), remapping ghost cells to their source (w_source). */
template <class R>
__device__ __forceinline__ void fetch_w(const Mh2dArgs<R> &a, const R *const *Win,
                                        const R *const *Uin, bool raw, int r, int c, R w[5])
{
    int rr, cc, neg;
    bool cons;
    w_source(a, raw, r, c, rr, cc, neg, cons);
    const long long idx = (long long) rr * a.pitch + cc;
    if (cons) {
        cons_to_prim_2d_guarded(a.gas, (R) a.vol, Uin[0][idx], Uin[1][idx], Uin[2][idx], Uin[3][idx], w);
        w[4] = sound_speed(a.gas, w[0], w[3]);
        return;
    }
#pragma unroll
    for (int q = 0; q < 5; q++) w[q] = Win[q][idx];
    if (neg == 1) w[1] = -w[1];
    if (neg == 2) w[2] = -w[2];
}

/* Asynchronous 4-byte global -> shared copies (cp.async, no register
 * staging), grouped per ring row: commit after a row's copies, wait until
 * at most N groups of this thread are still in flight. */
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned s = (unsigned) __cvta_generic_to_shared(smem);
    unsigned long long g;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(gmem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(g) : "memory");
}

__device__ __forceinline__ void cp_async_commit()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void record_error(HydroStepControl *ctrl, int code, int where)
{
    if (atomicCAS(&ctrl->error_code, 0, code) == 0) ctrl->error_cell = where;
}

/* Shared memory of one CTA: the W row ring and one batch of faces. */
template <class R, int NT>
struct Mh2dShared {
    /* rows in the ring: FP32 keeps a fourth so the row after next can be
     * copied in asynchronously while the current row is solved */
    static constexpr int RING = sizeof(R) == 4 ? 4 : 3;
    R ring[RING][5][NT + 2];    /* W rows (rho, u, v, p, a), columns c0-2 .. c0+NT-1 */
    R FL[4][2 * NT];            /* left face states; overwritten by the face flux */
    R FR[4][2 * NT];            /* right face states */
    R aL[2 * NT], aR[2 * NT];   /* sound speeds of the face states */
    R pg[2 * NT];               /* star-pressure guess (before the tol floor) */
    unsigned char reg[2 * NT];  /* PREG_* regime of each face */
    short listT[2 * NT];        /* faces needing the two-rarefaction guess */
    short listS[2 * NT];        /* faces needing the two-shock guess */
    int nT, nS;
    int item;
    int am_last;
    double red[2][NT / 32];
    /* FP64: the state each interior thread carries up its column (see
     * mh2d_item); FP32 keeps it in registers and these are unused */
    static constexpr int CQ = sizeof(R) == 8 ? 4 : 1;
    R ytop[CQ][NT];             /* low state of the y face above the current row */
    R gbot[CQ][NT];             /* update term of the y face below the current row */
};

/* The vacuum / vacuum-generation flux, out of line: rare, and kept out of
 * the finish loop's code. */
template <class R>
__device__ __noinline__ void vacuum_flux_dev(const GasConst<R> &c, R rl, R ul, R vl, R pl, R al,
                                             R rr, R ur, R vr, R pr, R ar, R F[4])
{
    hllc_vacuum_flux(c, rl, ul, vl, pl, al, rr, ur, vr, pr, ar, F);
}

/*
 * Solve faces 0..nF-1 of the batch in sm.FL / sm.FR (normal velocity in
 * slot 1) with the HLLC flux.  FP64: three dense passes over the CTA:
 * classify (sound speeds, vacuum test, guess regime), the expensive guesses
 * on compacted lists (two-rarefaction: three pow; two-shock: five divides
 * and two square roots), and the finish (wave speeds, S*, region flux).
 * Compaction keeps lanes busy where neighbouring faces fall into different
 * regimes, which the one-face-per-thread form serialises.  FP32: one pass,
 * one face per thread (the FP32 step batches only its x faces here; each y
 * face is solved in registers by its column's thread).  Its guesses are a
 * few approximate operations, and
 * the passes' shared-memory round trips and barriers cost more than the
 * divergence they avoid (2048^2 shear layer 14.5 -> 15.1 G cell-updates/s,
 * 8192^2 point blast 24.9 -> 27.6 G, the same results).  FP64: the
 * face's update term (flux * dt) * area replaces the left state in sm.FL
 * (faces [0, nXf) are x faces, area Ax, the rest y faces, Ay).  Both cells
 * of a face add or subtract this one product, so it is formed once per face;
 * the reference forms the same product for each cell (identical bits).
 * FP32: the flux itself, and each cell forms U + (F dt) A, which the FP32
 * build (contraction allowed) fuses; the point blast at 8192^2 needs that
 * accuracy near its vacuum.  Ends with a barrier.
 */
template <class R, int NT, bool TAPE = false>
__device__ __forceinline__ int solve_faces(Mh2dShared<R, NT> &sm, const GasConst<R> &gas, int nF,
                                           int nXf, R dtr, R Ax, R Ay,
                                           const TapeCtx<R> &tc = TapeCtx<R>{})
{
    const int tid = threadIdx.x;
    int err = DEV_OK;
    if constexpr (sizeof(R) == 4 && !TAPE) {
        for (int f = tid; f < nF; f += NT) {
            R F[4];
            const int rc = hllc_flux_2d(gas, sm.FL[0][f], sm.FL[1][f], sm.FL[2][f], sm.FL[3][f],
                                        sm.FR[0][f], sm.FR[1][f], sm.FR[2][f], sm.FR[3][f], F);
            if (rc) err = rc;
#pragma unroll
            for (int q = 0; q < 4; q++) sm.FL[q][f] = F[q];
        }
        __syncthreads();
        return err;
    } else {
        for (int f = tid; f < nF; f += NT) {
            R aL, aR, ppv;
            const int reg = hllc_classify(gas, sm.FL[0][f], sm.FL[1][f], sm.FL[3][f],
                                          sm.FR[0][f], sm.FR[1][f], sm.FR[3][f], aL, aR, ppv);
            sm.aL[f] = aL;
            sm.aR[f] = aR;
            sm.pg[f] = ppv;
            sm.reg[f] = (unsigned char) reg;
            if (reg == PREG_TRRS) sm.listT[atomicAdd(&sm.nT, 1)] = (short) f;
            else if (reg == PREG_TSRS) sm.listS[atomicAdd(&sm.nS, 1)] = (short) f;
        }
        __syncthreads();
        const int nT = sm.nT, nS = sm.nS;
        for (int i = tid; i < nT + nS; i += NT) {
            if constexpr (TAPE) {
                R z0, z1;
                int f;
                if (i < nT) {
                    f = sm.listT[i];
                    sm.pg[f] = guess_p_trrs_z(gas, sm.FL[1][f], sm.FL[3][f], sm.aL[f],
                                              sm.FR[1][f], sm.FR[3][f], sm.aR[f], z0, z1);
                } else {
                    f = sm.listS[i - nT];
                    sm.pg[f] = guess_p_tsrs_g(gas, sm.FL[0][f], sm.FL[1][f], sm.FL[3][f],
                                              sm.FR[0][f], sm.FR[1][f], sm.FR[3][f], sm.pg[f], z0, z1);
                }
                *tc.field(f, TAPE_Z0) = z0;
                *tc.field(f, TAPE_Z1) = z1;
            } else if (i < nT) {
                const int f = sm.listT[i];
                sm.pg[f] = guess_p_trrs(gas, sm.FL[1][f], sm.FL[3][f], sm.aL[f],
                                        sm.FR[1][f], sm.FR[3][f], sm.aR[f]);
            } else {
                const int f = sm.listS[i - nT];
                sm.pg[f] = guess_p_tsrs(gas, sm.FL[0][f], sm.FL[1][f], sm.FL[3][f],
                                        sm.FR[0][f], sm.FR[1][f], sm.FR[3][f], sm.pg[f]);
            }
        }
        __syncthreads();
        for (int f = tid; f < nF; f += NT) {
            R F[4];
            const R rl = sm.FL[0][f], ul = sm.FL[1][f], vl = sm.FL[2][f], pl = sm.FL[3][f];
            const R rr = sm.FR[0][f], ur = sm.FR[1][f], vr = sm.FR[2][f], pr = sm.FR[3][f];
            if constexpr (TAPE) {
                const R v[11] = { rl, ul, vl, pl, rr, ur, vr, pr, sm.aL[f], sm.aR[f], sm.pg[f] };
#pragma unroll
                for (int q = 0; q < 11; q++) *tc.field(f, q) = v[q];
                *tc.field(f, TAPE_REG) = (R) sm.reg[f];
            }
            if (sm.reg[f] == PREG_VACUUM) {
                vacuum_flux_dev(gas, rl, ul, vl, pl, sm.aL[f], rr, ur, vr, pr, sm.aR[f], F);
                if constexpr (TAPE) {
                    *tc.field(f, TAPE_QL) = R(0);
                    *tc.field(f, TAPE_QR) = R(0);
                    *tc.field(f, TAPE_SS) = R(0);
                }
            } else if constexpr (TAPE) {
                R wave[3];
                const int rc = hllc_finish(gas, rl, ul, vl, pl, sm.aL[f], rr, ur, vr, pr, sm.aR[f],
                                           sm.pg[f], F, wave);
                if (rc) err = rc;
                *tc.field(f, TAPE_QL) = wave[0];
                *tc.field(f, TAPE_QR) = wave[1];
                *tc.field(f, TAPE_SS) = wave[2];
            } else {
                const int rc = hllc_finish(gas, rl, ul, vl, pl, sm.aL[f], rr, ur, vr, pr, sm.aR[f],
                                           sm.pg[f], F);
                if (rc) err = rc;
            }
            if constexpr (sizeof(R) == 8) {
                const R A = (f < nXf) ? Ax : Ay;
#pragma unroll
                for (int q = 0; q < 4; q++) sm.FL[q][f] = (F[q] * dtr) * A;
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++) sm.FL[q][f] = F[q];
            }
        }
        __syncthreads();
        return err;
    }
}

/*
 * Process one work item (one strip of NT-2 columns x one chunk of chunk_h
 * rows) of step n with time step dt.  Shared by the single-grid and the
 * batched kernels; the caller reduces mx_x / mx_y and handles errors.
 */
template <class R, int LIM, int NT, int FIRST_ORDER, bool TAPE = false, bool GRAV = false>
__device__ __forceinline__ void mh2d_item(const Mh2dArgs<R> &a, Mh2dShared<R, NT> &sm, int item,
                                          long long n, double dt, double &mx_x, double &mx_y,
                                          int &err)
{
    const R dtr = (R) dt;
    /* a face's update term from what solve_faces left in sm.FL: FP64 stores
     * the term itself, FP32 the flux */
    auto upd = [&](R v, R area) -> R {
        if constexpr (sizeof(R) == 8) return v;
        else return (v * dtr) * area;
    };
    const R dtA_x = (R) (dt * a.area_x / a.vol);
    const R dtA_y = (R) (dt * a.area_y / a.vol);
    const R Ax = (R) a.area_x, Ay = (R) a.area_y;
    const int buf = (int) (n & 1);
    const bool raw = (n == 0);
    const R *const *Uin = a.U[buf];
    R *const *Uout = a.U[buf ^ 1];
    const R *const *Win = a.W[buf];
    R *const *Wout = a.W[buf ^ 1];
    const int tid = threadIdx.x;
    const int g = a.g, nx = a.nx, ny = a.ny;
    const int tx = nx + 2 * g, ty = ny + 2 * g;
    const int ymap[4] = { 0, 2, 1, 3 };   /* y fluxes come back as (mass, mom_y, mom_x, energy) */

    int strip, r_begin, r_end;
    mh2d_item_rows(a, item, strip, r_begin, r_end);
    const int c0 = g + strip * a.strip_w;
    const int sw = min(a.strip_w, nx - strip * a.strip_w);
    const int col = c0 - 1 + tid;
    const bool x_slot = tid <= sw + 1;
    const bool inner = tid >= 1 && tid <= sw;
    const bool ghost_xmin = (c0 == g) && tid == 0;
    const bool ghost_xmax = (c0 + sw == g + nx) && tid == sw + 1;
    const int nX = sw + 1;

    /* Rows inside [r_begin, r_end) need the strip plus two halo columns per
     * side (x work); rows outside need only the strip's own columns.  Cells
     * outside the padded grid (first order with one ghost layer) are never
     * read and are not loaded. */
    constexpr int RING = Mh2dShared<R, NT>::RING;
    auto load_row = [&](int r) {
        if (r < 0 || r >= ty) return;
        const bool full = (r >= r_begin && r < r_end);
        const int lo = full ? 0 : 2;
        const int hi = full ? sw + 3 : sw + 1;
        const int s = r % RING;
        for (int u = tid; u < NT + 2; u += NT) {
            const int c = c0 - 2 + u;
            if (u >= lo && u <= hi && c >= 0 && c < tx) {
                R w[5];
                fetch_w(a, Win, Uin, raw, r, c, w);
#pragma unroll
                for (int q = 0; q < 5; q++) sm.ring[s][q][u] = w[q];
            }
        }
    };

    /* FP32: the same row, with every cell that is a plain copy of a stored
     * cell (interior cells, periodic and mirror images without a sign
     * flip) copied by cp.async; the others are loaded as in load_row.
     * Always commits one group (possibly empty), so a wait for all but the
     * latest group means "all rows but the one issued last". */
    auto load_row_async = [&](int r) {
        if (r >= 0 && r < ty) {
            const bool full = (r >= r_begin && r < r_end);
            const int lo = full ? 0 : 2;
            const int hi = full ? sw + 3 : sw + 1;
            const int s = r % RING;
            for (int u = tid; u < NT + 2; u += NT) {
                const int c = c0 - 2 + u;
                if (u >= lo && u <= hi && c >= 0 && c < tx) {
                    int rr, cc, neg;
                    bool cons;
                    w_source(a, raw, r, c, rr, cc, neg, cons);
                    if (!cons && neg == 0) {
                        const long long idx = (long long) rr * a.pitch + cc;
#pragma unroll
                        for (int q = 0; q < 5; q++) cp_async4(&sm.ring[s][q][u], &Win[q][idx]);
                    } else {
                        R w[5];
                        fetch_w(a, Win, Uin, raw, r, c, w);
#pragma unroll
                        for (int q = 0; q < 5; q++) sm.ring[s][q][u] = w[q];
                    }
                }
            }
        }
        cp_async_commit();
    };

    /* y reconstruction of this thread's cell in row r, (rho, v, u, p) order */
    auto recon_y = [&](int r, R lo[4], R hi[4]) {
        const int u = tid + 1;
        const int sb = (r + RING - 1) % RING, sc = r % RING, st = (r + 1) % RING;
        const R rho = sm.ring[sc][0][u], vx = sm.ring[sc][1][u], vy = sm.ring[sc][2][u];
        const R p = sm.ring[sc][3][u], as = sm.ring[sc][4][u];
        if (FIRST_ORDER) {
            lo[0] = hi[0] = rho; lo[1] = hi[1] = vy; lo[2] = hi[2] = vx; lo[3] = hi[3] = p;
            return;
        }
        R d[4];
        d[0] = limit_slope<LIM>(rho - sm.ring[sb][0][u], sm.ring[st][0][u] - rho);
        const R dvx = limit_slope<LIM>(vx - sm.ring[sb][1][u], sm.ring[st][1][u] - vx);
        d[1] = limit_slope<LIM>(vy - sm.ring[sb][2][u], sm.ring[st][2][u] - vy);
        d[2] = dvx;
        d[3] = limit_slope<LIM>(p - sm.ring[sb][3][u], sm.ring[st][3][u] - p);
        hancock_2d(dtA_y, dv(dtA_y, rho), rho, vy, vx, p, as, d, dvx, lo, hi);
    };

    /* x reconstruction of slot tid in ring row s, (rho, u, v, p) order */
    auto recon_x = [&](int s, R lo[4], R hi[4]) {
        const int u = tid + 1;
        const R rho = sm.ring[s][0][u], vx = sm.ring[s][1][u], vy = sm.ring[s][2][u];
        const R p = sm.ring[s][3][u], as = sm.ring[s][4][u];
        if (FIRST_ORDER) {
            lo[0] = hi[0] = rho; lo[1] = hi[1] = vx; lo[2] = hi[2] = vy; lo[3] = hi[3] = p;
            return;
        }
        R d[4];
        d[0] = limit_slope<LIM>(rho - sm.ring[s][0][u - 1], sm.ring[s][0][u + 1] - rho);
        d[1] = limit_slope<LIM>(vx - sm.ring[s][1][u - 1], sm.ring[s][1][u + 1] - vx);
        d[2] = limit_slope<LIM>(vy - sm.ring[s][2][u - 1], sm.ring[s][2][u + 1] - vy);
        d[3] = limit_slope<LIM>(p - sm.ring[s][3][u - 1], sm.ring[s][3][u + 1] - p);
        hancock_2d(dtA_x, dv(dtA_x, rho), rho, vx, vy, p, as, d, d[1], lo, hi);
    };

    /* ---- prologue: the faces below r_begin ---- */
    load_row(r_begin - 2);
    load_row(r_begin - 1);
    load_row(r_begin);
    __syncthreads();
    /* What a thread carries up its column from row to row: ytop, the low
     * state of the y face above its cell (from the reconstruction one row
     * below), and gbot, the update term of the y face below.  FP64 keeps
     * them in shared memory: registers set the FP64 occupancy (128 per
     * thread at 4 CTAs per SM), and these eight doubles would stay live
     * across every out-of-line divide, square root and pow call of the face
     * solve (2048^2 shear layer: 1276 -> 1292 M cell-updates/s).  FP32 keeps
     * them in registers (11.73 against 11.65 G in shared memory). */
    constexpr bool CARRY_SMEM = sizeof(R) == 8;
    /* FP32 (no tape): each interior thread also solves the y face above its
     * cell itself, from the two states it holds in registers, so y faces
     * never pass through shared memory; only the x faces, whose states come
     * from two threads, are batched there */
    constexpr bool YREG = sizeof(R) == 4 && !TAPE;
    R ytop[4], gbot[4];         /* FP32 */
    R tmp_lo[4], prev_hi[4];
    if (inner) recon_y(r_begin - 1, tmp_lo, prev_hi);
    __syncthreads();
    load_row(r_begin + 1);
    if constexpr (RING == 4) load_row_async(r_begin + 2);
    if (tid == 0) { sm.nT = 0; sm.nS = 0; }
    __syncthreads();
    if constexpr (YREG) {
        /* FP32: the face below the chunk is solved by its column's thread */
        if (inner) {
            recon_y(r_begin, tmp_lo, ytop);
            const int rc = hllc_flux_2d(a.gas, prev_hi[0], prev_hi[1], prev_hi[2], prev_hi[3],
                                        tmp_lo[0], tmp_lo[1], tmp_lo[2], tmp_lo[3], gbot);
            if (rc) err = rc;
        }
        __syncthreads();
    } else {
        if (inner) {
            recon_y(r_begin, tmp_lo, ytop);
            if constexpr (CARRY_SMEM) {
#pragma unroll
                for (int q = 0; q < 4; q++) sm.ytop[q][tid] = ytop[q];
            }
#pragma unroll
            for (int q = 0; q < 4; q++) { sm.FL[q][tid - 1] = prev_hi[q]; sm.FR[q][tid - 1] = tmp_lo[q]; }
        }
        __syncthreads();
        {
            int rc;
            if constexpr (TAPE) {
                const TapeCtx<R> tc{ a.tape, a.tape_plane, a.pitch, 0, -1, r_begin - 1, c0 };
                rc = solve_faces<R, NT, true>(sm, a.gas, sw, 0, dtr, Ax, Ay, tc);
            } else {
                rc = solve_faces<R, NT>(sm, a.gas, sw, 0, dtr, Ax, Ay);
            }
            if (rc) err = rc;
        }
        if (inner) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if constexpr (CARRY_SMEM) sm.gbot[q][tid] = sm.FL[q][tid - 1];
                else gbot[q] = sm.FL[q][tid - 1];
            }
        }
        __syncthreads();
    }

    /* ---- march up the rows ---- */
    /* FP32: the item's maxima of a + |u| and a + |v| in float (a maximum of
     * floats is exact, and so is its conversion to double), merged into the
     * double maxima once per item instead of converting every cell's */
    float imx_x = -CUDART_INF_F, imx_y = -CUDART_INF_F;
    for (int r = r_begin; r < r_end; r++) {
        /* FP32: this row's U is loaded before the face solve, which hides its
         * latency (FP64 keeps those registers: its out-of-line divide, square
         * root and pow calls would carry them) */
        R upre[4];
        if constexpr (sizeof(R) == 4) {
            if (inner) {
                const long long pidx = (long long) r * a.pitch + col;
#pragma unroll
                for (int q = 0; q < 4; q++) upre[q] = Uin[q][pidx];
            }
        }
        if constexpr (RING == 4) {
            /* issue the row after next (the last one this item reads is
             * r_end + 1), then wait for row r + 2, issued one row ago */
            if (r + 3 <= r_end + 1) load_row_async(r + 3);
            else cp_async_commit();
            cp_async_wait<1>();
        } else {
            load_row(r + 2);
        }
        if (tid == 0) { sm.nT = 0; sm.nS = 0; }
        __syncthreads();

        R nhi[4];
        R gy[4];                /* FP32: the flux of the y face above this row */
        if (inner) {
            R nlo[4];
            recon_y(r + 1, nlo, nhi);
            /* the face above this row: low state carried from below, high
             * state from the cell above, whose own high state is carried to
             * the next row (FP64: now; FP32: after the update) */
            if constexpr (YREG) {
                const int rc = hllc_flux_2d(a.gas, ytop[0], ytop[1], ytop[2], ytop[3],
                                            nlo[0], nlo[1], nlo[2], nlo[3], gy);
                if (rc) err = rc;
            } else {
                const int f = nX + tid - 1;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if constexpr (CARRY_SMEM) {
                        sm.FL[q][f] = sm.ytop[q][tid];
                        sm.ytop[q][tid] = nhi[q];
                    } else {
                        sm.FL[q][f] = ytop[q];
                    }
                    sm.FR[q][f] = nlo[q];
                }
            }
        }
        if (x_slot) {
            R xl[4], xh[4];
            recon_x(r % RING, xl, xh);
            if (tid <= sw) {
#pragma unroll
                for (int q = 0; q < 4; q++) sm.FL[q][tid] = xh[q];
            }
            if (tid >= 1) {
#pragma unroll
                for (int q = 0; q < 4; q++) sm.FR[q][tid - 1] = xl[q];
            }
        }
        __syncthreads();
        {
            int rc;
            if constexpr (TAPE) {
                const TapeCtx<R> tc{ a.tape, a.tape_plane, a.pitch, nX, r, r, c0 };
                rc = solve_faces<R, NT, true>(sm, a.gas, nX + sw, nX, dtr, Ax, Ay, tc);
            } else {
                rc = solve_faces<R, NT>(sm, a.gas, YREG ? nX : nX + sw, nX, dtr, Ax, Ay);
            }
            if (rc) err = rc;
        }

        const long long rowbase = (long long) r * a.pitch;
        if (inner) {
            const long long idx = rowbase + col;
            R gtop[4];
#pragma unroll
            for (int q = 0; q < 4; q++) gtop[q] = YREG ? gy[q] : sm.FL[q][nX + tid - 1];
            R Un[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                R v;
                if constexpr (sizeof(R) == 4) v = upre[q];
                else v = Uin[q][idx];
                if constexpr (sizeof(R) == 8) {
                    v = v + sm.FL[q][tid - 1];
                    v = v - sm.FL[q][tid];
                    v = v + sm.gbot[ymap[q]][tid];
                    v = v - gtop[ymap[q]];
                } else {
                    v = v + (sm.FL[q][tid - 1] * dtr) * Ax;
                    v = v - (sm.FL[q][tid] * dtr) * Ax;
                    v = v + (gbot[ymap[q]] * dtr) * Ay;
                    v = v - (gtop[ymap[q]] * dtr) * Ay;
                }
                Un[q] = v;
                if constexpr (!GRAV) Uout[q][idx] = v;
            }
            if constexpr (GRAV) {
                /* gravity source, RK4 on energy (src/source_term.c:185-240) */
                gravity_kick((R) (-dt * a.gravity), Un[0], Un[2], Un[3]);
#pragma unroll
                for (int q = 0; q < 4; q++) Uout[q][idx] = Un[q];
            }
            R w[4];
            cons_to_prim_2d_guarded(a.gas, (R) a.vol, Un[0], Un[1], Un[2], Un[3], w);
            const R as = sound_speed(a.gas, w[0], w[3]);
#pragma unroll
            for (int q = 0; q < 4; q++) Wout[q][idx] = w[q];
            Wout[4][idx] = as;
            const R sx = as + fabs(w[1]);
            const R sy = as + fabs(w[2]);
            if constexpr (sizeof(R) == 4) {
                if (sx > imx_x) imx_x = sx;
                if (sy > imx_y) imx_y = sy;
            } else {
                /* FP64: the compares on the bits (integer pipe; IEEE order, NaN
                 * never larger, as with the FP64 compare) */
                if (lt(mx_x, sx)) mx_x = sx;
                if (lt(mx_y, sy)) mx_y = sy;
            }

            /* first ghost row below / above the domain: one-sided update */
            if (r == g) {
                const long long gi = idx - a.pitch;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    Uout[q][gi] = Uin[q][gi] - upd(CARRY_SMEM ? sm.gbot[ymap[q] % Mh2dShared<R, NT>::CQ][tid]
                                                              : gbot[ymap[q]], Ay);
            }
            if (r == g + ny - 1) {
                const long long gi = idx + a.pitch;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    Uout[q][gi] = Uin[q][gi] + upd(gtop[ymap[q]], Ay);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if constexpr (CARRY_SMEM) {
                    sm.gbot[q][tid] = gtop[q];
                } else {
                    ytop[q] = nhi[q];
                    gbot[q] = gtop[q];
                }
            }
        }
        /* first ghost column left / right of the domain */
        if (ghost_xmin) {
            const long long gi = rowbase + col;
#pragma unroll
            for (int q = 0; q < 4; q++) Uout[q][gi] = Uin[q][gi] - upd(sm.FL[q][0], Ax);
        }
        if (ghost_xmax) {
            const long long gi = rowbase + col;
#pragma unroll
            for (int q = 0; q < 4; q++) Uout[q][gi] = Uin[q][gi] + upd(sm.FL[q][sw], Ax);
        }
        __syncthreads();
    }
    if constexpr (RING == 4) cp_async_wait<0>();   /* nothing in flight into the next item's ring */
    if constexpr (sizeof(R) == 4) {
        if ((double) imx_x > mx_x) mx_x = (double) imx_x;
        if ((double) imx_y > mx_y) mx_y = (double) imx_y;
    }
}

/*
 * One time step of one grid.  The grid is persistent: each CTA takes
 * (strip, row chunk) items from a device counter until none are left, so
 * SMs that finish early take more work (the FP64 pipe of an SM is shared by
 * its CTAs).
 */
template <class R, int LIM, int NT, int FIRST_ORDER, bool TAPE = false, bool GRAV = false>
__global__ void __launch_bounds__(NT, (sizeof(R) == 4 ? MH2D_CTAS_FP32 : MH2D_CTAS_FP64))
mh2d_step_kernel(const Mh2dArgs<R> a)
{
    static_assert(NT % 32 == 0, "NT must be a whole number of warps");
    HydroStepControl *ctrl = a.ctrl;
    if (!*(volatile int *) &ctrl->active) return;

    /* ---- dt for this step (src/integrator_muscl_hancock.c:533-549) ---- */
    const long long n = ctrl->num_steps;
    const double t_now = ctrl->t;
    const double Sx = from_ordered_bits(ctrl->smax[n % 3][0]);
    const double Sy = from_ordered_bits(ctrl->smax[n % 3][1]);
    const double cfl = (n < a.sp.shrink_steps) ? a.sp.cfl_shrunk : a.sp.cfl;
    double dt = cfl / (Sx / a.dx + Sy / a.dy);
    const double tf = ctrl->tf;
    if (t_now + dt > tf) dt = tf - t_now;
    if (dt == 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctrl->dt = dt;
            record_error(ctrl, DEV_ERR_DT_ZERO, -1);
            ctrl->active = 0;
        }
        return;
    }

    __shared__ Mh2dShared<R, NT> sm;
    const int tid = threadIdx.x;
    const int n_items = mh2d_n_items(a);
    double mx_x = -CUDART_INF, mx_y = -CUDART_INF;
    int err = DEV_OK;

    for (;;) {
        if (tid == 0) sm.item = atomicAdd(&ctrl->work_next, 1);
        __syncthreads();
        const int item = sm.item;
        __syncthreads();
        if (item >= n_items) break;
        mh2d_item<R, LIM, NT, FIRST_ORDER, TAPE, GRAV>(a, sm, item, n, dt, mx_x, mx_y, err);
    }

    if (err) record_error(ctrl, err, (int) blockIdx.x);

    /* ---- CTA maxima -> device maxima for the next step's dt ---- */
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ox = __shfl_xor_sync(0xffffffffu, mx_x, o);
        const double oy = __shfl_xor_sync(0xffffffffu, mx_y, o);
        if (ox > mx_x) mx_x = ox;
        if (oy > mx_y) mx_y = oy;
    }
    if ((tid & 31) == 0) {
        sm.red[0][tid >> 5] = mx_x;
        sm.red[1][tid >> 5] = mx_y;
    }
    __syncthreads();
    if (tid == 0) {
        double bx = sm.red[0][0], by = sm.red[1][0];
        for (int w = 1; w < NT / 32; w++) {
            if (sm.red[0][w] > bx) bx = sm.red[0][w];
            if (sm.red[1][w] > by) by = sm.red[1][w];
        }
        const int nxt = (int) ((n + 1) % 3);
        atomicMax(&ctrl->smax[nxt][0], ordered_bits(bx));
        atomicMax(&ctrl->smax[nxt][1], ordered_bits(by));
        __threadfence();
        sm.am_last = (atomicAdd(&ctrl->blocks_done, 1u) == gridDim.x - 1);
    }
    __syncthreads();

    /* ---- last CTA: advance the clock (src/integrator_muscl_hancock.c:1143-1154) ---- */
    if (sm.am_last && tid == 0) {
        __threadfence();
        volatile HydroStepControl *vc = ctrl;
        ctrl->dt = dt;
        ctrl->work_next = 0;
        if (vc->error_code != 0) {
            ctrl->active = 0;
        } else {
            const double tn = t_now + dt;
            const long long nn = n + 1;
            ctrl->t = tn;
            ctrl->num_steps = nn;
            const int nn2 = (int) ((n + 2) % 3);
            ctrl->smax[nn2][0] = ordered_bits(-CUDART_INF);
            ctrl->smax[nn2][1] = ordered_bits(-CUDART_INF);
            int act = (tn < tf) && (vc->max_steps < 0 || nn < vc->max_steps);
            if (a.sp.is_storing &&
                tn >= a.sp.storing_interval *
                          (double) (vc->store_count - a.sp.store_initial_offset + 1)) {
                ctrl->snapshot_due = 1;
                act = 0;
            }
            ctrl->active = act;
        }
        ctrl->blocks_done = 0;
    }
}

/* ------------------------------------------------------------------ */
/* Batched ensembles: many independent grids in one launch per step.   */
/* ------------------------------------------------------------------ */

/* Work queue of one batched step launch. */
struct HydroBatchControl {
    int work_next;           /* next global work item */
    unsigned int ctas_done;  /* CTAs that left the queue (last one resets both) */
};

template <class R>
struct Mh2dBatchArgs {
    const Mh2dArgs<R> *inst;  /* per-instance arguments (device memory), each with its own control */
    const int *item_off;      /* n_inst + 1 prefix offsets of the instances' work items */
    int n_inst;
    int total_items;
    HydroBatchControl *bctrl;
};

/* dt of instance `a` for its current step, or 0 when it must not step
 * (inactive; on dt == 0 the error is recorded as the single-grid kernel does). */
template <class R>
__device__ double instance_dt(const Mh2dArgs<R> &a, long long &n)
{
    HydroStepControl *ctrl = a.ctrl;
    if (!*(volatile int *) &ctrl->active) return 0.0;
    n = ctrl->num_steps;
    const double t_now = ctrl->t;
    const double Sx = from_ordered_bits(ctrl->smax[n % 3][0]);
    const double Sy = from_ordered_bits(ctrl->smax[n % 3][1]);
    const double cfl = (n < a.sp.shrink_steps) ? a.sp.cfl_shrunk : a.sp.cfl;
    double dt = cfl / (Sx / a.dx + Sy / a.dy);
    const double tf = ctrl->tf;
    if (t_now + dt > tf) dt = tf - t_now;
    if (dt == 0.0) {
        ctrl->dt = dt;
        record_error(ctrl, DEV_ERR_DT_ZERO, -1);
        ctrl->active = 0;
    }
    return dt;
}

/* Clock advance of one instance by the last of its items (the single-grid
 * kernel's last-CTA block, per instance). */
__device__ __forceinline__ void instance_bookkeeping(HydroStepControl *ctrl, const HydroStepParams &sp,
                                                     long long n, double dt)
{
    volatile HydroStepControl *vc = ctrl;
    ctrl->dt = dt;
    if (vc->error_code != 0) {
        ctrl->active = 0;
    } else {
        const double tn = vc->t + dt;
        const long long nn = n + 1;
        ctrl->t = tn;
        ctrl->num_steps = nn;
        const int nn2 = (int) ((n + 2) % 3);
        ctrl->smax[nn2][0] = ordered_bits(-CUDART_INF);
        ctrl->smax[nn2][1] = ordered_bits(-CUDART_INF);
        int act = (tn < vc->tf) && (vc->max_steps < 0 || nn < vc->max_steps);
        if (sp.is_storing &&
            tn >= sp.storing_interval * (double) (vc->store_count - sp.store_initial_offset + 1)) {
            ctrl->snapshot_due = 1;
            act = 0;
        }
        ctrl->active = act;
    }
    ctrl->blocks_done = 0;
}

/*
 * One time step of every active instance of a batch.  Persistent CTAs take
 * global items from one queue; an item belongs to one instance (found by
 * binary search in the prefix offsets), whose dt the CTA derives from that
 * instance's control block.  After each item the CTA folds its CFL maxima
 * into the instance's next-step words, and the instance's last item
 * advances that instance's clock.  Instances are laid out largest first,
 * so the queue drains the big grids early and the tail is made of small
 * items.
 */
template <class R, int LIM, int NT, int FIRST_ORDER>
__global__ void __launch_bounds__(NT, (sizeof(R) == 4 ? MH2D_CTAS_FP32 : MH2D_CTAS_FP64))
mh2d_batch_step_kernel(const Mh2dBatchArgs<R> b)
{
    __shared__ Mh2dShared<R, NT> sm;
    __shared__ int s_inst, s_local, s_go, s_last;
    __shared__ long long s_n;
    __shared__ double s_dt;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) {
            const int gi = atomicAdd(&b.bctrl->work_next, 1);
            s_go = 0;
            sm.item = gi;
            if (gi < b.total_items) {
                int lo = 0, hi = b.n_inst - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (b.item_off[mid] <= gi) lo = mid;
                    else hi = mid - 1;
                }
                s_inst = lo;
                s_local = gi - b.item_off[lo];
                long long n = 0;
                const double dt = instance_dt(b.inst[lo], n);
                s_dt = dt;
                s_n = n;
                s_go = (dt != 0.0);
            }
        }
        __syncthreads();
        if (sm.item >= b.total_items) break;
        const int go = s_go, inst = s_inst, local = s_local;
        const long long n = s_n;
        const double dt = s_dt;
        __syncthreads();
        if (!go) continue;
        const Mh2dArgs<R> &a = b.inst[inst];
        double mx_x = -CUDART_INF, mx_y = -CUDART_INF;
        int err = DEV_OK;
        mh2d_item<R, LIM, NT, FIRST_ORDER>(a, sm, local, n, dt, mx_x, mx_y, err);
        if (err) record_error(a.ctrl, err, inst);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ox = __shfl_xor_sync(0xffffffffu, mx_x, o);
            const double oy = __shfl_xor_sync(0xffffffffu, mx_y, o);
            if (ox > mx_x) mx_x = ox;
            if (oy > mx_y) mx_y = oy;
        }
        if ((tid & 31) == 0) {
            sm.red[0][tid >> 5] = mx_x;
            sm.red[1][tid >> 5] = mx_y;
        }
        __syncthreads();
        if (tid == 0) {
            double bx = sm.red[0][0], by = sm.red[1][0];
            for (int w = 1; w < NT / 32; w++) {
                if (sm.red[0][w] > bx) bx = sm.red[0][w];
                if (sm.red[1][w] > by) by = sm.red[1][w];
            }
            HydroStepControl *ctrl = a.ctrl;
            const int nxt = (int) ((n + 1) % 3);
            atomicMax(&ctrl->smax[nxt][0], ordered_bits(bx));
            atomicMax(&ctrl->smax[nxt][1], ordered_bits(by));
            __threadfence();
            const int n_items = b.item_off[inst + 1] - b.item_off[inst];
            s_last = (atomicAdd(&ctrl->blocks_done, 1u) == (unsigned) (n_items - 1));
            if (s_last) {
                __threadfence();
                instance_bookkeeping(ctrl, a.sp, n, dt);
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&b.bctrl->ctas_done, 1u) == gridDim.x - 1) {
            b.bctrl->work_next = 0;
            b.bctrl->ctas_done = 0;
        }
    }
}

}  // namespace hydro

#endif
