// FP64 Crank-Nicolson / Jacobi-COCG time stepper: one persistent cooperative
// kernel integrates a whole signal.
//
// Reference: MRI_simulation.solve (DmriFemLib.py:878-915).  Each step of the
// reference assembles A = M/k + F(f(t)) and b = L(u, f(tp)) and calls a PETSc
// Krylov solver (DmriFemLib.py:901-907).  In complex form (u = ur + i ui,
// duplicated interface dofs) the step is
//     (A_re + i cn J_g) u_new = (B_re - i co J_g) u_old
//     A_re = M/k + theta (K + T + R),  B_re = M/k - (1 - theta)(K + T + R),
//     cn = theta q f(t),  co = (1 - theta) q f(tp),
// complex symmetric, so it is solved with COCG (CG with the unconjugated
// bilinear form) and the Jacobi preconditioner diag(A)^-1.
//
// Layout: the matrix lives in sliced ELL (32 rows per slice, column-major in a
// slice) packed per signal as double2 {A_re, J_g} plus B_re, so a warp reads
// 32 consecutive 16-byte entries per column step (coalesced 128-bit loads).
// Vectors are double2 (re, im) of length n_pad = 32 * slices.
//
// One kernel runs all steps and iterations; phases are separated by a bounded
// grid barrier (bt_common.cuh).  GB300 executes FP64 at a small fraction of
// its FP32 rate, so the loop is arranged to minimise FP64 operations:
//   * q = A p is carried by the recurrence q = A z + beta q (p = z + beta p),
//     so the only SpMV of an iteration is A z: 4 FP64 FMAs per stored entry;
//   * the Jacobi inverse D^-1 = 1 / (A_re,ii + i cn J_ii) is formed once per
//     step (phase R), not per iteration;
//   * the initial guess extrapolates the last steps' states in time (up to
//     fourth order: x0 = u_n + 4 d_1 - 6 d_2 + 4 d_3 - d_4 with d_j =
//     u_{n-j+1} - u_{n-j}), and A x0 is formed from stored per-row products
//     A_re d_j, J_g d_j of earlier steps, so phase R gathers u_n only.  On the
//     40^3 two-compartment workload the order-4 guess needs about 30% fewer
//     COCG iterations than the linear one.
// Per iteration (two barriers):
//   phase A:  w = A z ; q = w + beta q ; p = z + beta p ; mu = p^T q   | barrier
//   phase B:  x += alpha p ; r -= alpha q ; z = D^-1 r ; rho = r^T z  | barrier
// The three solution levels u_{n-1}, u_n, u_{n+1} rotate through three
// buffers so that phase R can gather u_{n-1} and u_n while writing u_{n+1}.
// Reductions are per-block partials summed by every block in block order, so
// all blocks take identical decisions and results are bitwise reproducible.
#include "bt_common.cuh"

#include <algorithm>
#include <cmath>

namespace bt {

constexpr int kThreads64 = 256;
constexpr int kRed = 1 + kMaxCompartments;  // reduction width of the signal phase

struct Solver64 {
    int64_t n_pad = 0, sell = 0;
    int32_t nblocks = 0;
    DevBuf<double2> aj;          // SELL {A_re, J_g}
    DevBuf<double> bre;          // SELL B_re
    DevBuf<double> dA, dJ, w;    // per row
    DevBuf<int32_t> rcomp;       // compartment per row (-1 padding)
    DevBuf<double2> u[3], r, z, p, q, dinv;
    DevBuf<double2> pa, pj, hd;  // extrapolated guess: previous products and the ring of differences
    DevBuf<double> partials;
    DevBuf<unsigned> bar;
    DevBuf<int> status;
    DevBuf<double> cn, co, relres, out;
    DevBuf<double> ps;           // q F(tp) per step (pseudo-periodic phase)
    DevBuf<int32_t> iters;
    DevBuf<double> gq;           // gradient direction for the pack kernel
    DevBuf<double2> saved;       // final solutions [nsig][n_pad]
    int32_t saved_nsig = 0;
    // two signals a launch (k_step64_pair): [row][2] vectors, per-signal schedules and results
    DevBuf<double2> pu[3], pr, pz, pp, pq, pdinv, ppa, ppj, phd;
    DevBuf<double> pcn, pco, prelres, pout, ppartials;
    DevBuf<int32_t> piters;
    int32_t pair_blocks = 0;
    int32_t pair_variant = 0;
};

struct StepArgs {
    int32_t n_slices;
    const int32_t* __restrict__ sl_ptr;
    const int32_t* __restrict__ sl_w;
    const int32_t* __restrict__ col;
    const double2* __restrict__ aj;
    const double* __restrict__ bre;
    const double* __restrict__ dA;
    const double* __restrict__ dJ;
    const double* __restrict__ w;
    const int32_t* __restrict__ rcomp;
    double2* u0;
    double2* u1;
    double2* u2;
    double2* r;
    double2* z;
    double2* p;
    double2* q;
    double2* dinv;
    double* partials;
    unsigned* bar;
    int* status;
    const double* __restrict__ cn;
    const double* __restrict__ co;
    int32_t n_steps;
    int32_t maxit;
    int32_t nc;
    int32_t extrapolate;
    double rtol2;
    const double* __restrict__ rhs_vec;  // nullable: right-hand side b = rhs_vec (real) for step 0
    const double2* __restrict__ extra;   // nullable: extra[step * n_pad + i] added to b at every step
    // pseudo-periodic boundary term (nullable per_ptr): b_i += (1 - theta) sum_e
    // val.c exp(i ps[step] g.(val.x, val.y, val.z)) u_n[col[e]]
    const int32_t* __restrict__ per_ptr;
    const int32_t* __restrict__ per_col;
    const PerVal* __restrict__ per_val;
    const double* __restrict__ per_ps;
    const double* __restrict__ g3;
    double theta;
    int64_t n_rows;
    double2* save;                       // nullable: state after step s saved to save[(s+1)/save_every - 1]
    int32_t save_every;
    int64_t n_pad;
    int32_t* iters;
    double* relres;
    double* out;
    // extrapolated initial guess: per row, the products A_re u, J_g u of the
    // previous step's u_n (pa, pj) and a ring of four (d_j, A_re d_j, J_g d_j)
    double2* pa;
    double2* pj;
    double2* hd;                         // [4][3][n_pad]
    unsigned long long wait_ns;          // time limit of every grid-wide wait
    int32_t stall;                       // failure-detection hook: the first wait runs out (stalled_wait)
};

// Grid-wide deterministic sum of NV doubles: block partials go to one of two
// alternating buffers (a block may start the next reduction while a slower
// block is still reading the previous one), then every block adds the
// partials in block order.  On return every thread holds the sums in v[].
template <int NV>
__device__ __forceinline__ bool reduce_all(double (&v)[NV], double* partials, unsigned nb, unsigned& flip,
                                           unsigned* bar, int* status, unsigned& gen, double* sm,
                                           double* red, unsigned long long wait_ns) {
    block_sum<NV>(v, sm);
    double* P = partials + (size_t)(flip & 1u) * nb * kRed;
    ++flip;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) P[blockIdx.x * kRed + k] = v[k];
    }
    if (!grid_barrier(bar, nb, status, gen, wait_ns)) return false;
    if ((threadIdx.x >> 5) == 0) {
        const int lane = threadIdx.x & 31;
        double t[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) t[k] = 0.0;
        for (unsigned b = lane; b < nb; b += 32) {
#pragma unroll
            for (int k = 0; k < NV; ++k) t[k] += __ldcg(&P[b * kRed + k]);
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) t[k] = warp_sum(t[k]);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) red[k] = t[k];
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = red[k];
    __syncthreads();
    return true;
}

// Coefficient of d_j in the order-h extrapolation x0 = u_n + sum_j c_j d_j:
// (-1)^(j+1) C(h, j) for 1 <= j <= h <= 4.
__device__ __forceinline__ double extrap_coef(int h, int j) {
    const double b = (j == 1 || j == h - 1) ? (double)h : (j == h ? 1.0 : 6.0);
    return (j & 1) ? b : -b;
}

__global__ void __launch_bounds__(kThreads64) k_step64(StepArgs a) {
    __shared__ double sm[32 * kRed];
    __shared__ double red[kRed];
    const int lane = threadIdx.x & 31;
    const int warps_per_block = kThreads64 / 32;
    const int gw = blockIdx.x * warps_per_block + (threadIdx.x >> 5);
    const int total_warps = gridDim.x * warps_per_block;
    const unsigned nb = gridDim.x;
    unsigned gen = 0, flip = 0;
    double2* U[3] = {a.u0, a.u1, a.u2};
    double2* x = U[1];
    if (a.stall) {   // bar[2] is never written: the wait runs out and the launch ends with DEV_TIMEOUT
        stalled_wait(a.bar + 2, a.status, a.wait_ns);
        return;
    }

    for (int step = 0; step < a.n_steps; ++step) {
        const double cn = a.cn[step], co = a.co[step];
        const double2* __restrict__ cur = U[step % 3];
        const double2* __restrict__ prev = U[(step + 2) % 3];
        x = U[(step + 1) % 3];
        // ---- phase R: b = (B_re - i co J) u_n ; x = 2 u_n - u_{n-1} ;
        //               r = b - A x ; D^-1 ; z = D^-1 r
        double acc[4] = {0.0, 0.0, 0.0, 0.0};  // rho.re, rho.im, |r|^2, |b|^2
        // extrapolation order of this step: the history holds `step` differences
        const int h = (a.rhs_vec && step == 0) ? 0 : min(step, a.extrapolate);
        for (int s = gw; s < a.n_slices; s += total_warps) {
            const int32_t base = a.sl_ptr[s], wdt = a.sl_w[s];
            double2 sA = make_double2(0.0, 0.0), sJ = sA, sB = sA;
            for (int k = 0; k < wdt; ++k) {
                const int32_t e = base + k * 32 + lane;
                const int32_t c = a.col[e];
                const double2 m = a.aj[e];
                const double br = a.bre[e];
                const double2 uj = cur[c];
                sA.x = fma(m.x, uj.x, sA.x); sA.y = fma(m.x, uj.y, sA.y);
                sJ.x = fma(m.y, uj.x, sJ.x); sJ.y = fma(m.y, uj.y, sJ.y);
                sB.x = fma(br, uj.x, sB.x);  sB.y = fma(br, uj.y, sB.y);
            }
            const int64_t i = (int64_t)s * 32 + lane;
            double2 b = (a.rhs_vec && step == 0) ? make_double2(a.rhs_vec[i], 0.0)
                                                 : make_double2(fma(co, sJ.y, sB.x), fma(-co, sJ.x, sB.y));
            if (a.extra) {
                const double2 ex2 = a.extra[(int64_t)step * a.n_pad + i];
                b.x += ex2.x;
                b.y += ex2.y;
            }
            if (a.per_ptr && i < a.n_rows) {
                const int32_t e0 = a.per_ptr[i], e1 = a.per_ptr[i + 1];
                if (e0 < e1) {
                    const double ps = a.per_ps[step];
                    const double g0 = a.g3[0], g1 = a.g3[1], g2 = a.g3[2];
                    double2 acc2 = make_double2(0.0, 0.0);
                    for (int32_t e = e0; e < e1; ++e) {
                        const PerVal v = a.per_val[e];
                        double sn, cs;
                        sincos(ps * (g0 * v.x + g1 * v.y + g2 * v.z), &sn, &cs);
                        const double2 uk = cur[a.per_col[e]];
                        acc2.x = fma(v.c, cs * uk.x - sn * uk.y, acc2.x);
                        acc2.y = fma(v.c, sn * uk.x + cs * uk.y, acc2.y);
                    }
                    b.x = fma(1.0 - a.theta, acc2.x, b.x);
                    b.y = fma(1.0 - a.theta, acc2.y, b.y);
                }
            }
            // x0 = u_n + sum_j c_j d_j and A x0 from the stored products (binomial
            // extrapolation of order h: c = (1), (2,-1), (3,-3,1), (4,-6,4,-1))
            const double2 ui = cur[i];
            double2 gA = sA, gJ = sJ, xi = ui;
            if (step >= 1 && a.extrapolate > 0) {
                // this step's difference d_1 = u_n - u_{n-1} and its products enter the ring
                const double2 vi = prev[i], pA = a.pa[i], pJ = a.pj[i];
                double2* H = a.hd + (size_t)(step & 3) * 3 * a.n_pad;
                H[i] = make_double2(ui.x - vi.x, ui.y - vi.y);
                H[a.n_pad + i] = make_double2(sA.x - pA.x, sA.y - pA.y);
                H[2 * a.n_pad + i] = make_double2(sJ.x - pJ.x, sJ.y - pJ.y);
            }
            if (a.extrapolate > 0) {
                a.pa[i] = sA;
                a.pj[i] = sJ;
            }
            for (int j = 1; j <= h; ++j) {
                const double c = extrap_coef(h, j);
                const double2* H = a.hd + (size_t)((step - j + 1) & 3) * 3 * a.n_pad;
                const double2 d = H[i], dA = H[a.n_pad + i], dJ = H[2 * a.n_pad + i];
                xi.x = fma(c, d.x, xi.x); xi.y = fma(c, d.y, xi.y);
                gA.x = fma(c, dA.x, gA.x); gA.y = fma(c, dA.y, gA.y);
                gJ.x = fma(c, dJ.x, gJ.x); gJ.y = fma(c, dJ.y, gJ.y);
            }
            const double2 ax = make_double2(fma(-cn, gJ.y, gA.x), fma(cn, gJ.x, gA.y));
            x[i] = xi;
            const double2 rr = make_double2(b.x - ax.x, b.y - ax.y);
            const double2 di = cinv(make_double2(a.dA[i], cn * a.dJ[i]));
            const double2 zz = cmul(di, rr);
            a.dinv[i] = di;
            a.r[i] = rr;
            a.z[i] = zz;
            a.p[i] = make_double2(0.0, 0.0);
            a.q[i] = make_double2(0.0, 0.0);
            const double2 rz = cmul(rr, zz);
            acc[0] += rz.x;
            acc[1] += rz.y;
            acc[2] += rr.x * rr.x + rr.y * rr.y;
            acc[3] += b.x * b.x + b.y * b.y;
        }
        if (!reduce_all<4>(acc, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
        double2 rho = make_double2(acc[0], acc[1]);
        double rr2 = acc[2];
        const double bb2 = acc[3];
        const double tol2 = a.rtol2 * bb2;
        double2 beta = make_double2(0.0, 0.0);
        int it = 0;
        bool failed = false;  // uniform across the grid: every block sees the same sums
        while (rr2 > tol2) {
            if (it >= a.maxit) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
                failed = true;
                break;
            }
            // ---- phase A: w = A z ; q = w + beta q ; p = z + beta p ; mu = p^T q
            double mu[2] = {0.0, 0.0};
            for (int s = gw; s < a.n_slices; s += total_warps) {
                const int32_t base = a.sl_ptr[s], wdt = a.sl_w[s];
                double2 sA = make_double2(0.0, 0.0), sJ = sA;
                int k = 0;
                // four independent neighbour gathers in flight per thread
                for (; k + 4 <= wdt; k += 4) {
                    int32_t cc[4];
                    double2 mm[4], zz[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int32_t e = base + (k + u) * 32 + lane;
                        cc[u] = a.col[e];
                        mm[u] = a.aj[e];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) zz[u] = a.z[cc[u]];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        sA.x = fma(mm[u].x, zz[u].x, sA.x); sA.y = fma(mm[u].x, zz[u].y, sA.y);
                        sJ.x = fma(mm[u].y, zz[u].x, sJ.x); sJ.y = fma(mm[u].y, zz[u].y, sJ.y);
                    }
                }
                for (; k < wdt; ++k) {
                    const int32_t e = base + k * 32 + lane;
                    const double2 m = a.aj[e];
                    const double2 zc = a.z[a.col[e]];
                    sA.x = fma(m.x, zc.x, sA.x); sA.y = fma(m.x, zc.y, sA.y);
                    sJ.x = fma(m.y, zc.x, sJ.x); sJ.y = fma(m.y, zc.y, sJ.y);
                }
                const int64_t i = (int64_t)s * 32 + lane;
                const double2 zi = a.z[i], pi = a.p[i], qo = a.q[i];
                const double2 bp = cmul(beta, pi), bq = cmul(beta, qo);
                const double2 pn = make_double2(zi.x + bp.x, zi.y + bp.y);
                const double2 qn = make_double2(fma(-cn, sJ.y, sA.x) + bq.x, fma(cn, sJ.x, sA.y) + bq.y);
                a.p[i] = pn;
                a.q[i] = qn;
                const double2 pq = cmul(pn, qn);
                mu[0] += pq.x;
                mu[1] += pq.y;
            }
            if (!reduce_all<2>(mu, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
            const double2 muv = make_double2(mu[0], mu[1]);
            const double mun = muv.x * muv.x + muv.y * muv.y;
            if (!(mun > 0.0) || !isfinite(mun)) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_BREAKDOWN);
                failed = true;
                break;
            }
            const double2 alpha = cdiv(rho, muv);
            // ---- phase B: x += alpha p ; r -= alpha q ; z = D^-1 r
            double acc3[3] = {0.0, 0.0, 0.0};
            for (int s = gw; s < a.n_slices; s += total_warps) {
                const int64_t i = (int64_t)s * 32 + lane;
                const double2 pn = a.p[i], qi = a.q[i];
                double2 xi = x[i], ri = a.r[i];
                const double2 ap = cmul(alpha, pn), aq = cmul(alpha, qi);
                xi.x += ap.x; xi.y += ap.y;
                ri.x -= aq.x; ri.y -= aq.y;
                const double2 zi = cmul(a.dinv[i], ri);
                x[i] = xi;
                a.r[i] = ri;
                a.z[i] = zi;
                const double2 rz = cmul(ri, zi);
                acc3[0] += rz.x;
                acc3[1] += rz.y;
                acc3[2] += ri.x * ri.x + ri.y * ri.y;
            }
            if (!reduce_all<3>(acc3, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
            const double2 rho_new = make_double2(acc3[0], acc3[1]);
            rr2 = acc3[2];
            ++it;
            const double rhon = rho.x * rho.x + rho.y * rho.y;
            if (!(rhon > 0.0) || !isfinite(rr2)) {
                if (rr2 > tol2 || !isfinite(rr2)) {
                    if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_BREAKDOWN);
                    failed = true;
                }
                break;
            }
            beta = cdiv(rho_new, rho);
            rho = rho_new;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.iters[step] = it;
            a.relres[step] = (bb2 > 0.0) ? sqrt(rr2 / bb2) : sqrt(rr2);
        }
        if (failed) return;
        // The last phase B (or phase R when no iteration ran) ended in a grid
        // barrier, so u_{n+1} is complete before the next phase R gathers it.
        if (a.save && ((step + 1) % a.save_every) == 0) {
            double2* dst = a.save + (int64_t)((step + 1) / a.save_every - 1) * a.n_pad;
            for (int s = gw; s < a.n_slices; s += total_warps) {
                const int64_t i = (int64_t)s * 32 + lane;
                dst[i] = x[i];
            }
        }
    }
    // ---- signal: S = sum w Re(u_N), per compartment
    double acc[kRed];
#pragma unroll
    for (int k = 0; k < kRed; ++k) acc[k] = 0.0;
    for (int s = gw; s < a.n_slices; s += total_warps) {
        const int64_t i = (int64_t)s * 32 + lane;
        const int c = a.rcomp[i];
        if (c >= 0) {
            const double v = a.w[i] * x[i].x;
            acc[0] += v;
#pragma unroll
            for (int k = 0; k < kMaxCompartments; ++k)
                if (k == c) acc[1 + k] += v;
        }
    }
    if (!reduce_all<kRed>(acc, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
    if (blockIdx.x == 0 && threadIdx.x < kRed) a.out[threadIdx.x] = red[threadIdx.x];
}

// ------------------------------------------------------ two signals a launch --
// Two signals of one gradient direction share A_re and J_g (only cn, co differ),
// so one launch can step both: a thread loads a row's column indices and matrix
// values once for the pair, its neighbour gathers fetch both signals' values from
// one 32-byte pair slot ([row][signal] interleaved vectors), and the pair's grid
// reductions share one set of barriers.  Each signal keeps its own COCG scalars
// and stopping test; a converged signal's vectors stay untouched (uniform branch,
// the sums are grid-identical) while the other one iterates.  The per-row
// arithmetic of a signal is that of k_step64 in the same order.
struct PairArgs {
    int32_t n_slices;
    const int32_t* __restrict__ sl_ptr;
    const int32_t* __restrict__ sl_w;
    const int32_t* __restrict__ col;
    const double2* __restrict__ aj;
    const double* __restrict__ bre;
    const double* __restrict__ dA;
    const double* __restrict__ dJ;
    const double* __restrict__ w;
    const int32_t* __restrict__ rcomp;
    double2* u0;                         // vectors: [row][2], length 2 n_pad
    double2* u1;
    double2* u2;
    double2* r;
    double2* z;
    double2* p;
    double2* q;
    double2* dinv;
    double2* pa;
    double2* pj;
    double2* hd;                         // [4][3][2 n_pad]
    double* partials;
    unsigned* bar;
    int* status;
    const double* __restrict__ cn;       // [2][n_steps]
    const double* __restrict__ co;       // [2][n_steps]
    int32_t n_steps;
    int32_t maxit;
    int32_t extrapolate;
    double rtol2;
    int64_t n_pad;
    int32_t* iters;                      // [2][n_steps]
    double* relres;                      // [2][n_steps]
    double* out;                         // [2][kRed]
    unsigned long long wait_ns;
    int32_t stall;
};

// w = A z for one row of the signals J0 .. J0 + NJ - 1 of the pair (sA = A_re z,
// sJ = J_g z), four neighbour rows in flight as in k_step64's phase A.
template <int J0, int NJ>
__device__ __forceinline__ void pair_row_spmv(const int32_t* __restrict__ col, const double2* __restrict__ aj,
                                              const double2* z, int32_t base, int32_t wdt, int lane,
                                              double2 (&sA)[2], double2 (&sJ)[2]) {
    int k = 0;
    for (; k + 4 <= wdt; k += 4) {
        int32_t cc[4];
        double2 mm[4], zz[4][NJ];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int32_t e = base + (k + u) * 32 + lane;
            cc[u] = col[e];
            mm[u] = aj[e];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < NJ; ++j) zz[u][j] = z[2 * (size_t)cc[u] + J0 + j];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
                double2& A = sA[J0 + j];
                double2& J = sJ[J0 + j];
                A.x = fma(mm[u].x, zz[u][j].x, A.x); A.y = fma(mm[u].x, zz[u][j].y, A.y);
                J.x = fma(mm[u].y, zz[u][j].x, J.x); J.y = fma(mm[u].y, zz[u][j].y, J.y);
            }
    }
    for (; k < wdt; ++k) {
        const int32_t e = base + k * 32 + lane;
        const double2 m = aj[e];
        const size_t c2 = 2 * (size_t)col[e];
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const double2 zc = z[c2 + J0 + j];
            double2& A = sA[J0 + j];
            double2& J = sJ[J0 + j];
            A.x = fma(m.x, zc.x, A.x); A.y = fma(m.x, zc.y, A.y);
            J.x = fma(m.y, zc.x, J.x); J.y = fma(m.y, zc.y, J.y);
        }
    }
}

// MINB blocks per SM: 2 caps the registers at 128 (a few spilled) so that one
// thread per row fits the grid; 1 leaves ~200 registers and a warp takes two
// slices.
template <int MINB>
__global__ void __launch_bounds__(kThreads64, MINB) k_step64_pair(PairArgs a) {
    __shared__ double sm[32 * kRed];
    __shared__ double red[kRed];
    const int lane = threadIdx.x & 31;
    const int warps_per_block = kThreads64 / 32;
    const int gw = blockIdx.x * warps_per_block + (threadIdx.x >> 5);
    const int total_warps = gridDim.x * warps_per_block;
    const unsigned nb = gridDim.x;
    const size_t hs = (size_t)2 * a.n_pad;   // length of one pair vector
    unsigned gen = 0, flip = 0;
    double2* U[3] = {a.u0, a.u1, a.u2};
    double2* x = U[1];
    if (a.stall) {
        stalled_wait(a.bar + 2, a.status, a.wait_ns);
        return;
    }

    for (int step = 0; step < a.n_steps; ++step) {
        const double cn[2] = {a.cn[step], a.cn[a.n_steps + step]};
        const double co[2] = {a.co[step], a.co[a.n_steps + step]};
        const double2* __restrict__ cur = U[step % 3];
        const double2* __restrict__ prev = U[(step + 2) % 3];
        x = U[(step + 1) % 3];
        // ---- phase R (per signal as in k_step64): b, extrapolated x0, r, D^-1, z
        double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // per signal: rho.re, rho.im, |r|^2, |b|^2
        const int h = min(step, a.extrapolate);
        for (int s = gw; s < a.n_slices; s += total_warps) {
            const int32_t base = a.sl_ptr[s], wdt = a.sl_w[s];
            double2 sA[2], sJ[2], sB[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) sA[j] = sJ[j] = sB[j] = make_double2(0.0, 0.0);
            for (int k = 0; k < wdt; ++k) {
                const int32_t e = base + k * 32 + lane;
                const size_t c2 = 2 * (size_t)a.col[e];
                const double2 m = a.aj[e];
                const double br = a.bre[e];
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const double2 uj = cur[c2 + j];
                    sA[j].x = fma(m.x, uj.x, sA[j].x); sA[j].y = fma(m.x, uj.y, sA[j].y);
                    sJ[j].x = fma(m.y, uj.x, sJ[j].x); sJ[j].y = fma(m.y, uj.y, sJ[j].y);
                    sB[j].x = fma(br, uj.x, sB[j].x);  sB[j].y = fma(br, uj.y, sB[j].y);
                }
            }
            const int64_t i = (int64_t)s * 32 + lane;
            const double dAi = a.dA[i], dJi = a.dJ[i];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const size_t vi = 2 * (size_t)i + j;
                const double2 b = make_double2(fma(co[j], sJ[j].y, sB[j].x), fma(-co[j], sJ[j].x, sB[j].y));
                const double2 ui = cur[vi];
                double2 gA = sA[j], gJ = sJ[j], xi = ui;
                if (step >= 1 && a.extrapolate > 0) {
                    const double2 uo = prev[vi], pA = a.pa[vi], pJ = a.pj[vi];
                    double2* H = a.hd + (size_t)(step & 3) * 3 * hs;
                    H[vi] = make_double2(ui.x - uo.x, ui.y - uo.y);
                    H[hs + vi] = make_double2(sA[j].x - pA.x, sA[j].y - pA.y);
                    H[2 * hs + vi] = make_double2(sJ[j].x - pJ.x, sJ[j].y - pJ.y);
                }
                if (a.extrapolate > 0) {
                    a.pa[vi] = sA[j];
                    a.pj[vi] = sJ[j];
                }
                for (int jj = 1; jj <= h; ++jj) {
                    const double c = extrap_coef(h, jj);
                    const double2* H = a.hd + (size_t)((step - jj + 1) & 3) * 3 * hs;
                    const double2 d = H[vi], dAv = H[hs + vi], dJv = H[2 * hs + vi];
                    xi.x = fma(c, d.x, xi.x); xi.y = fma(c, d.y, xi.y);
                    gA.x = fma(c, dAv.x, gA.x); gA.y = fma(c, dAv.y, gA.y);
                    gJ.x = fma(c, dJv.x, gJ.x); gJ.y = fma(c, dJv.y, gJ.y);
                }
                const double2 ax = make_double2(fma(-cn[j], gJ.y, gA.x), fma(cn[j], gJ.x, gA.y));
                x[vi] = xi;
                const double2 rr = make_double2(b.x - ax.x, b.y - ax.y);
                const double2 di = cinv(make_double2(dAi, cn[j] * dJi));
                const double2 zz = cmul(di, rr);
                a.dinv[vi] = di;
                a.r[vi] = rr;
                a.z[vi] = zz;
                a.p[vi] = make_double2(0.0, 0.0);
                a.q[vi] = make_double2(0.0, 0.0);
                const double2 rz = cmul(rr, zz);
                acc[4 * j + 0] += rz.x;
                acc[4 * j + 1] += rz.y;
                acc[4 * j + 2] += rr.x * rr.x + rr.y * rr.y;
                acc[4 * j + 3] += b.x * b.x + b.y * b.y;
            }
        }
        if (!reduce_all<8>(acc, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
        double2 rho[2], beta[2];
        double rr2[2], bb2[2], tol2[2];
        int it[2] = {0, 0};
        bool act[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            rho[j] = make_double2(acc[4 * j], acc[4 * j + 1]);
            rr2[j] = acc[4 * j + 2];
            bb2[j] = acc[4 * j + 3];
            tol2[j] = a.rtol2 * bb2[j];
            beta[j] = make_double2(0.0, 0.0);
            act[j] = rr2[j] > tol2[j];
        }
        bool failed = false;  // uniform across the grid, as every decision below
        while (act[0] || act[1]) {
            if ((act[0] && it[0] >= a.maxit) || (act[1] && it[1] >= a.maxit)) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
                failed = true;
                break;
            }
            // ---- phase A: w = A z ; q = w + beta q ; p = z + beta p ; mu = p^T q
            double mu[4] = {0.0, 0.0, 0.0, 0.0};
            for (int s = gw; s < a.n_slices; s += total_warps) {
                const int32_t base = a.sl_ptr[s], wdt = a.sl_w[s];
                double2 sA[2], sJ[2];
#pragma unroll
                for (int j = 0; j < 2; ++j) sA[j] = sJ[j] = make_double2(0.0, 0.0);
                if (act[0] && act[1])
                    pair_row_spmv<0, 2>(a.col, a.aj, a.z, base, wdt, lane, sA, sJ);
                else if (act[0])
                    pair_row_spmv<0, 1>(a.col, a.aj, a.z, base, wdt, lane, sA, sJ);
                else
                    pair_row_spmv<1, 1>(a.col, a.aj, a.z, base, wdt, lane, sA, sJ);
                const int64_t i = (int64_t)s * 32 + lane;
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    if (!act[j]) continue;
                    const size_t vi = 2 * (size_t)i + j;
                    const double2 zi = a.z[vi], pi = a.p[vi], qo = a.q[vi];
                    const double2 bp = cmul(beta[j], pi), bq = cmul(beta[j], qo);
                    const double2 pn = make_double2(zi.x + bp.x, zi.y + bp.y);
                    const double2 qn = make_double2(fma(-cn[j], sJ[j].y, sA[j].x) + bq.x,
                                                    fma(cn[j], sJ[j].x, sA[j].y) + bq.y);
                    a.p[vi] = pn;
                    a.q[vi] = qn;
                    const double2 pq = cmul(pn, qn);
                    mu[2 * j] += pq.x;
                    mu[2 * j + 1] += pq.y;
                }
            }
            if (!reduce_all<4>(mu, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
            double2 alpha[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                alpha[j] = make_double2(0.0, 0.0);
                if (!act[j]) continue;
                const double2 muv = make_double2(mu[2 * j], mu[2 * j + 1]);
                const double mun = muv.x * muv.x + muv.y * muv.y;
                if (!(mun > 0.0) || !isfinite(mun)) failed = true;
                else alpha[j] = cdiv(rho[j], muv);
            }
            if (failed) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_BREAKDOWN);
                break;
            }
            // ---- phase B: x += alpha p ; r -= alpha q ; z = D^-1 r
            double acc3[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            for (int s = gw; s < a.n_slices; s += total_warps) {
                const int64_t i = (int64_t)s * 32 + lane;
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    if (!act[j]) continue;
                    const size_t vi = 2 * (size_t)i + j;
                    const double2 pn = a.p[vi], qi = a.q[vi];
                    double2 xi = x[vi], ri = a.r[vi];
                    const double2 ap = cmul(alpha[j], pn), aq = cmul(alpha[j], qi);
                    xi.x += ap.x; xi.y += ap.y;
                    ri.x -= aq.x; ri.y -= aq.y;
                    const double2 zi = cmul(a.dinv[vi], ri);
                    x[vi] = xi;
                    a.r[vi] = ri;
                    a.z[vi] = zi;
                    const double2 rz = cmul(ri, zi);
                    acc3[3 * j] += rz.x;
                    acc3[3 * j + 1] += rz.y;
                    acc3[3 * j + 2] += ri.x * ri.x + ri.y * ri.y;
                }
            }
            if (!reduce_all<6>(acc3, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                if (!act[j]) continue;
                const double2 rho_new = make_double2(acc3[3 * j], acc3[3 * j + 1]);
                rr2[j] = acc3[3 * j + 2];
                ++it[j];
                const double rhon = rho[j].x * rho[j].x + rho[j].y * rho[j].y;
                if (!(rhon > 0.0) || !isfinite(rr2[j])) {
                    if (rr2[j] > tol2[j] || !isfinite(rr2[j])) failed = true;
                    act[j] = false;
                    continue;
                }
                beta[j] = cdiv(rho_new, rho[j]);
                rho[j] = rho_new;
                act[j] = rr2[j] > tol2[j];
            }
            if (failed) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_BREAKDOWN);
                break;
            }
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                a.iters[j * a.n_steps + step] = it[j];
                a.relres[j * a.n_steps + step] = (bb2[j] > 0.0) ? sqrt(rr2[j] / bb2[j]) : sqrt(rr2[j]);
            }
        }
        if (failed) return;
    }
    // ---- signals: S_j = sum w Re(u_N,j), per compartment
    for (int j = 0; j < 2; ++j) {
        double acc[kRed];
#pragma unroll
        for (int k = 0; k < kRed; ++k) acc[k] = 0.0;
        for (int s = gw; s < a.n_slices; s += total_warps) {
            const int64_t i = (int64_t)s * 32 + lane;
            const int c = a.rcomp[i];
            if (c >= 0) {
                const double v = a.w[i] * x[2 * (size_t)i + j].x;
                acc[0] += v;
#pragma unroll
                for (int k = 0; k < kMaxCompartments; ++k)
                    if (k == c) acc[1 + k] += v;
            }
        }
        if (!reduce_all<kRed>(acc, a.partials, nb, flip, a.bar, a.status, gen, sm, red, a.wait_ns)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
#pragma unroll
            for (int k = 0; k < kRed; ++k) a.out[j * kRed + k] = acc[k];
        }
    }
}

// Initial state of a pair: both signals start from u0 (or 1); padding rows 0.
__global__ void k_pair_init(int64_t n, int64_t n_pad, const int32_t* __restrict__ dof_vertex,
                            const double* __restrict__ u0, double2* __restrict__ x, double2* __restrict__ xprev) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    const double2 v = (i < n) ? make_double2(u0 ? u0[dof_vertex[i]] : 1.0, 0.0) : make_double2(0.0, 0.0);
    x[2 * i] = v;
    x[2 * i + 1] = v;
    xprev[2 * i] = v;
    xprev[2 * i + 1] = v;
}

// Final states of a pair, [row][2] -> two [row] vectors.
__global__ void k_pair_extract(int64_t n_pad, const double2* __restrict__ x, double2* __restrict__ s0,
                               double2* __restrict__ s1) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    s0[i] = x[2 * i];
    s1[i] = x[2 * i + 1];
}

// Pack the SELL values of one signal: {A_re, J_g}, B_re, and the diagonals.
__global__ void k_pack64(int64_t sell, const int32_t* __restrict__ sl_pos, const double* __restrict__ M,
                         const double* __restrict__ K, const double* __restrict__ T, const double* __restrict__ R,
                         const double* __restrict__ Jx, const double* __restrict__ Jy,
                         const double* __restrict__ Jz, const double* __restrict__ g, double inv_k,
                         double theta, const double* __restrict__ PB, double2* __restrict__ aj,
                         double* __restrict__ bre) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= sell) return;
    const int32_t p = sl_pos[e];
    if (p < 0) {
        aj[e] = make_double2(0.0, 0.0);
        bre[e] = 0.0;
        return;
    }
    const double mk = M[p] * inv_k;
    const double S = K[p] + T[p] + R[p];
    aj[e] = make_double2(mk + theta * (PB ? S + PB[p] : S), g[0] * Jx[p] + g[1] * Jy[p] + g[2] * Jz[p]);
    bre[e] = mk - (1.0 - theta) * S;
}

__global__ void k_rows64(int64_t n, int64_t n_pad, const int32_t* __restrict__ diag_pos,
                         const double* __restrict__ M, const double* __restrict__ K, const double* __restrict__ T,
                         const double* __restrict__ R, const double* __restrict__ Jx,
                         const double* __restrict__ Jy, const double* __restrict__ Jz,
                         const double* __restrict__ g, double inv_k, double theta, const double* __restrict__ PB,
                         const double* __restrict__ wsrc, const int32_t* __restrict__ comp,
                         const int32_t* __restrict__ dof_vertex, const double* __restrict__ u0,
                         double* __restrict__ dA, double* __restrict__ dJ, double* __restrict__ w,
                         int32_t* __restrict__ rcomp, double2* __restrict__ x, double2* __restrict__ xprev,
                         double2* __restrict__ pa) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    if (i < n) {
        const int32_t p = diag_pos[i];
        dA[i] = M[p] * inv_k + theta * (K[p] + T[p] + R[p] + (PB ? PB[p] : 0.0));
        dJ[i] = g[0] * Jx[p] + g[1] * Jy[p] + g[2] * Jz[p];
        w[i] = wsrc[i];
        rcomp[i] = comp[i];
        x[i] = make_double2(u0 ? u0[dof_vertex[i]] : 1.0, 0.0);
        xprev[i] = x[i];
    } else {
        dA[i] = 1.0;
        dJ[i] = 0.0;
        w[i] = 0.0;
        rcomp[i] = -1;
        x[i] = make_double2(0.0, 0.0);
        xprev[i] = x[i];
    }
    pa[i] = make_double2(0.0, 0.0);
}

static void map_status(int st) {
    switch (st) {
        case DEV_OK: return;
        case DEV_TIMEOUT: throw Error(BT_ERR_TIMEOUT, "stepper: a grid barrier wait ran out of time");
        case DEV_NOT_CONVERGED: throw Error(BT_ERR_NOT_CONVERGED, "stepper: COCG reached max_iterations");
        case DEV_BREAKDOWN: throw Error(BT_ERR_BREAKDOWN, "stepper: COCG breakdown (p^T A p = 0)");
        default: throw Error(BT_ERR_CUDA, "stepper: device status " + std::to_string(st));
    }
}

// Allocate the FP64 workspace for a mesh and a schedule of n_steps.
static void prepare_fp64(bt_ctx* ctx, Solver64& W) {
    Mesh& m = ctx->mesh;
    Schedule& S = ctx->sched;
    W.n_pad = (int64_t)m.n_slices * 32;
    W.sell = m.sell_entries;
    W.aj.alloc(W.sell);
    W.bre.alloc(W.sell);
    W.dA.alloc(W.n_pad); W.dJ.alloc(W.n_pad); W.w.alloc(W.n_pad);
    W.rcomp.alloc(W.n_pad);
    for (auto* v : {&W.u[0], &W.u[1], &W.u[2], &W.r, &W.z, &W.p, &W.q, &W.dinv}) v->alloc(W.n_pad);
    W.bar.alloc(3);   // [0] arrivals, [1] generation, [2] never written (stalled_wait)
    W.pa.alloc(W.n_pad);
    W.pj.alloc(W.n_pad);
    W.hd.alloc((size_t)12 * W.n_pad);
    W.status.alloc(1);
    W.cn.alloc(S.n_steps); W.co.alloc(S.n_steps);
    W.relres.alloc(S.n_steps);
    W.iters.alloc(S.n_steps);
    W.out.alloc(kRed);
    W.gq.alloc(3);
    int per_sm = 0;
    BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step64, kThreads64, 0));
    BT_REQUIRE(per_sm >= 1, BT_ERR_CUDA, "stepper kernel does not fit on an SM");
    const int need = (m.n_slices + kThreads64 / 32 - 1) / (kThreads64 / 32);
    // With fewer blocks a warp takes two or more slices and each grid barrier
    // has fewer arrivals and pollers.  On GB300 one block per SM is faster
    // while the mesh needs at most four blocks per SM of one thread per row
    // (40^3: 1.19x, 48^3: 1.15x), equal beyond (64^3, 311 k rows: 0.6 %
    // slower), so "auto" caps there only.  (Loading the block partials of a
    // grid sum with all threads of a block instead of one warp was 1.3 %
    // slower: the gain is not in the partial sums.)
    const int cap = ctx->opt_fp64_blocks_per_sm > 0 ? ctx->opt_fp64_blocks_per_sm
                    : (ctx->opt_fp64_blocks_per_sm < 0 && need <= 4 * ctx->num_sms) ? 1 : 0;
    if (cap > 0) per_sm = std::min(per_sm, cap);
    W.nblocks = std::max(1, std::min(per_sm * ctx->num_sms, need));
    W.partials.alloc((size_t)2 * W.nblocks * kRed);
}

// Pack the matrix of one signal (direction g, theta, dt), the row data, and the
// initial state u0 into u[0] and u[2] (so the first step does not extrapolate).
static void pack_signal_fp64(bt_ctx* ctx, Solver64& W, const double* gdir, const double* d_u0) {
    Mesh& m = ctx->mesh;
    Assembled& A = ctx->mat;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    const double inv_k = 1.0 / S.dt;
    W.gq.upload(gdir, 3, s);
    const double* PB = ctx->per.on ? ctx->per.PB.p : nullptr;
    k_pack64<<<(unsigned)((W.sell + 255) / 256), 256, 0, s>>>(W.sell, m.sl_pos, A.M, A.K, A.T, A.R, A.Jx, A.Jy,
                                                             A.Jz, W.gq, inv_k, S.theta, PB, W.aj, W.bre);
    k_rows64<<<(unsigned)((W.n_pad + 255) / 256), 256, 0, s>>>(
        m.n_dofs, W.n_pad, m.diag_pos, A.M, A.K, A.T, A.R, A.Jx, A.Jy, A.Jz, W.gq, inv_k, S.theta, PB, A.w, m.dof_comp,
        m.dof_vertex, d_u0, W.dA, W.dJ, W.w, W.rcomp, W.u[0], W.u[2], W.u[1]);
    BT_CUDA(cudaGetLastError());
}

// One cooperative launch of k_step64 over n_steps steps with the schedule
// d_cn[0..n_steps), d_co[...]; the state enters in u[0] (u[2] = previous
// level) and leaves in u[n_steps % 3].  Returns the launch's device time.
static float run_steps_fp64(bt_ctx* ctx, Solver64& W, const double* d_cn, const double* d_co, int n_steps,
                            bool extrapolate, const double* rhs_vec, double2* save, int save_every, double rtol,
                            int maxit, std::vector<int32_t>* iters_out, std::vector<double>* relres_out,
                            double* out_sig, const double2* extra = nullptr) {
    Mesh& m = ctx->mesh;
    cudaStream_t s = ctx->stream;
    W.bar.zero(s);
    W.status.zero(s);
    StepArgs a;
    a.n_slices = m.n_slices;
    a.sl_ptr = m.sl_ptr; a.sl_w = m.sl_w; a.col = m.sl_col;
    a.aj = W.aj; a.bre = W.bre; a.dA = W.dA; a.dJ = W.dJ; a.w = W.w; a.rcomp = W.rcomp;
    a.u0 = W.u[0]; a.u1 = W.u[1]; a.u2 = W.u[2];
    a.r = W.r; a.z = W.z; a.p = W.p; a.q = W.q; a.dinv = W.dinv;
    a.partials = W.partials; a.bar = W.bar; a.status = W.status;
    a.cn = d_cn; a.co = d_co;
    a.n_steps = n_steps;
    a.maxit = maxit;
    a.nc = m.n_comp;
    a.extrapolate = extrapolate ? std::max(1, std::min(4, ctx->opt_fp64_extrapolate)) : 0;
    a.pa = W.pa;
    a.pj = W.pj;
    a.hd = W.hd;
    a.rtol2 = rtol * rtol;
    a.rhs_vec = rhs_vec;
    a.extra = extra;
    const Periodic& P = ctx->per;
    a.per_ptr = P.on ? P.ptr.p : nullptr;
    a.per_col = P.col.p;
    a.per_val = P.val.p;
    a.per_ps = W.ps.p;
    a.g3 = W.gq.p;
    a.theta = ctx->sched.theta;
    a.n_rows = m.n_dofs;
    if (P.on) BT_REQUIRE(W.ps.p && W.ps.n >= (size_t)n_steps, BT_ERR_STATE, "periodic phase schedule missing");
    a.save = save;
    a.save_every = save_every > 0 ? save_every : 1;
    a.n_pad = W.n_pad;
    a.iters = W.iters; a.relres = W.relres; a.out = W.out;
    a.wait_ns = ctx->opt_wait_ns;
    a.stall = ctx->opt_stall_first_wait;
    {
        const void* need_ptrs[] = {a.sl_ptr, a.sl_w, a.col, a.aj, a.bre, a.dA, a.dJ, a.w, a.rcomp, a.u0, a.u1,
                                   a.u2, a.r, a.z, a.p, a.q, a.dinv, a.partials, a.bar, a.status, a.cn, a.co,
                                   a.iters, a.relres, a.out};
        for (const void* ptr : need_ptrs)
            BT_REQUIRE(ptr != nullptr, BT_ERR_STATE, "stepper: a device buffer is not allocated");
        BT_REQUIRE(n_steps >= 1 && (size_t)n_steps <= W.iters.n, BT_ERR_INVALID, "stepper: bad step count");
    }
    void* args[] = {&a};
    BT_CUDA(cudaEventRecord(ctx->ev1, s));
    BT_CUDA(cudaLaunchCooperativeKernel((const void*)k_step64, dim3(W.nblocks), dim3(kThreads64), args, 0, s));
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    int hst = 0;
    BT_CUDA(cudaMemcpyAsync(&hst, W.status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (iters_out) {
        iters_out->resize(n_steps);
        W.iters.download(iters_out->data(), n_steps, s);
    }
    if (relres_out) {
        relres_out->resize(n_steps);
        W.relres.download(relres_out->data(), n_steps, s);
    }
    if (out_sig) W.out.download(out_sig, kRed, s);
    BT_CUDA(cudaStreamSynchronize(s));
    map_status(hst);
    float ms = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2));
    return ms;
}

// The paired kernel of option fp64.pair_signals: 1 = two blocks per SM, 2 = one.
static const void* pair_kernel(const bt_ctx* ctx) {
    return ctx->opt_fp64_pair == 2 ? (const void*)k_step64_pair<1> : (const void*)k_step64_pair<2>;
}

// Workspace of k_step64_pair (allocated on first use, kept across solves of one size).
static void prepare_pair(bt_ctx* ctx, Solver64& W) {
    const size_t n2 = (size_t)2 * W.n_pad;
    const size_t ns2 = (size_t)2 * ctx->sched.n_steps;
    for (auto* v : {&W.pu[0], &W.pu[1], &W.pu[2], &W.pr, &W.pz, &W.pp, &W.pq, &W.pdinv, &W.ppa, &W.ppj})
        v->alloc(n2);
    W.phd.alloc(12 * n2);
    W.pcn.alloc(ns2);
    W.pco.alloc(ns2);
    W.prelres.alloc(ns2);
    W.piters.alloc(ns2);
    W.pout.alloc(2 * kRed);
    int per_sm = 0;
    BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pair_kernel(ctx), kThreads64, 0));
    BT_REQUIRE(per_sm >= 1, BT_ERR_CUDA, "paired stepper kernel does not fit on an SM");
    W.pair_variant = ctx->opt_fp64_pair;
    const int need = (ctx->mesh.n_slices + kThreads64 / 32 - 1) / (kThreads64 / 32);
    W.pair_blocks = std::max(1, std::min(per_sm * ctx->num_sms, need));
    W.ppartials.alloc((size_t)2 * W.pair_blocks * kRed);
}

// One cooperative launch of k_step64_pair over the whole schedule for the two
// signals whose schedules are in W.pcn / W.pco (signal j at [j * n_steps]); the
// matrix and row data are those of pack_signal_fp64.  Returns the device time.
static float run_pair_fp64(bt_ctx* ctx, Solver64& W, const double* d_u0, double rtol, int maxit,
                           std::vector<int32_t>& iters, std::vector<double>& relres, double* out) {
    Mesh& m = ctx->mesh;
    cudaStream_t s = ctx->stream;
    const int n_steps = ctx->sched.n_steps;
    k_pair_init<<<(unsigned)((W.n_pad + 255) / 256), 256, 0, s>>>(m.n_dofs, W.n_pad, m.dof_vertex, d_u0,
                                                                   W.pu[0], W.pu[2]);
    BT_CUDA(cudaGetLastError());
    W.bar.zero(s);
    W.status.zero(s);
    PairArgs a;
    a.n_slices = m.n_slices;
    a.sl_ptr = m.sl_ptr; a.sl_w = m.sl_w; a.col = m.sl_col;
    a.aj = W.aj; a.bre = W.bre; a.dA = W.dA; a.dJ = W.dJ; a.w = W.w; a.rcomp = W.rcomp;
    a.u0 = W.pu[0]; a.u1 = W.pu[1]; a.u2 = W.pu[2];
    a.r = W.pr; a.z = W.pz; a.p = W.pp; a.q = W.pq; a.dinv = W.pdinv;
    a.pa = W.ppa; a.pj = W.ppj; a.hd = W.phd;
    a.partials = W.ppartials; a.bar = W.bar; a.status = W.status;
    a.cn = W.pcn; a.co = W.pco;
    a.n_steps = n_steps;
    a.maxit = maxit;
    a.extrapolate = ctx->opt_fp64_extrapolate != 0 ? std::max(1, std::min(4, ctx->opt_fp64_extrapolate)) : 0;
    a.rtol2 = rtol * rtol;
    a.n_pad = W.n_pad;
    a.iters = W.piters; a.relres = W.prelres; a.out = W.pout;
    a.wait_ns = ctx->opt_wait_ns;
    a.stall = ctx->opt_stall_first_wait;
    {
        const void* need_ptrs[] = {a.sl_ptr, a.sl_w, a.col, a.aj, a.bre, a.dA, a.dJ, a.w, a.rcomp, a.u0, a.u1,
                                   a.u2, a.r, a.z, a.p, a.q, a.dinv, a.pa, a.pj, a.hd, a.partials, a.bar,
                                   a.status, a.cn, a.co, a.iters, a.relres, a.out};
        for (const void* ptr : need_ptrs)
            BT_REQUIRE(ptr != nullptr, BT_ERR_STATE, "paired stepper: a device buffer is not allocated");
        BT_REQUIRE(n_steps >= 1 && W.pcn.n == (size_t)2 * n_steps && W.piters.n == (size_t)2 * n_steps,
                   BT_ERR_STATE, "paired stepper: schedule size mismatch");
    }
    void* args[] = {&a};
    BT_CUDA(cudaEventRecord(ctx->ev1, s));
    BT_CUDA(cudaLaunchCooperativeKernel(pair_kernel(ctx), dim3(W.pair_blocks), dim3(kThreads64), args, 0, s));
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    int hst = 0;
    BT_CUDA(cudaMemcpyAsync(&hst, W.status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    iters.resize((size_t)2 * n_steps);
    relres.resize((size_t)2 * n_steps);
    W.piters.download(iters.data(), iters.size(), s);
    W.prelres.download(relres.data(), relres.size(), s);
    W.pout.download(out, 2 * kRed, s);
    BT_CUDA(cudaStreamSynchronize(s));
    map_status(hst);
    float ms = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2));
    return ms;
}

static void schedule_row(const Schedule& S, int32_t row, double q, std::vector<double>& hcn,
                         std::vector<double>& hco) {
    BT_REQUIRE(row >= 0 && row < S.n_seq, BT_ERR_INVALID, "sequence index out of range");
    const double* fn = S.f_new.data() + (size_t)row * S.n_steps;
    const double* fo = S.f_old.data() + (size_t)row * S.n_steps;
    hcn.resize(S.n_steps);
    hco.resize(S.n_steps);
    for (int k = 0; k < S.n_steps; ++k) {
        hcn[k] = S.theta * q * fn[k];
        hco[k] = (1.0 - S.theta) * q * fo[k];
    }
}

void solve_fp64(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq,
                const double* u0, double rtol, int32_t maxit, double* sig, double* comp_sig, bt_stats* st) {
    Mesh& m = ctx->mesh;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    if (!ctx->s64) ctx->s64 = new Solver64();
    Solver64& W = *ctx->s64;
    prepare_fp64(ctx, W);
    W.saved.alloc((size_t)nsig * W.n_pad);
    W.saved_nsig = nsig;
    DevBuf<double> d_u0;
    if (u0) d_u0.upload(u0, m.n_v, s);
    std::vector<double> hcn, hco, hps, hout(kRed), hres;
    std::vector<int32_t> hit;
    ctx->last_iters.assign((size_t)nsig * S.n_steps, 0);
    if (st) {
        st->steps = S.n_steps;
        st->max_iterations = 0;
        st->total_iterations = 0;
        st->max_rel_residual = 0.0;
        st->refinements = 0;
        st->graph_launches = 0;
        st->kernel_launches = 0;
        st->stepper_ms = 0.0;
    }
    float stepper_ms_total = 0.0f;
    auto record = [&](int32_t sg, const double* out, const int32_t* it, const double* res) {
        sig[sg] = out[0];
        if (comp_sig)
            for (int c = 0; c < m.n_comp; ++c) comp_sig[(size_t)sg * m.n_comp + c] = out[1 + c];
        for (int k = 0; k < S.n_steps; ++k) {
            ctx->last_iters[(size_t)sg * S.n_steps + k] = it[k];
            if (st) {
                st->max_iterations = std::max(st->max_iterations, it[k]);
                st->total_iterations += it[k];
                st->max_rel_residual = std::max(st->max_rel_residual, res[k]);
            }
        }
    };
    // Two signals of one direction (identical gdir rows) share a k_step64_pair
    // launch: each signal is paired with the next unpaired signal of its
    // direction; outputs keep the call's order.
    std::vector<int32_t> mate(nsig, -1);
    if (ctx->opt_fp64_pair && !ctx->per.on) {
        for (int32_t i = 0; i < nsig; ++i) {
            if (mate[i] != -1) continue;
            const double* gi = gdir + 3 * i;
            for (int32_t j = i + 1; j < nsig; ++j) {
                const double* gj = gdir + 3 * j;
                if (mate[j] == -1 && gi[0] == gj[0] && gi[1] == gj[1] && gi[2] == gj[2]) {
                    mate[i] = j;
                    mate[j] = i;
                    break;
                }
            }
        }
    }
    BT_CUDA(cudaEventRecord(ctx->ev0, s));
    for (int32_t sg = 0; sg < nsig; ++sg) {
        if (mate[sg] >= 0 && mate[sg] < sg) continue;   // stepped with its earlier partner
        if (mate[sg] > sg) {
            const int32_t idx[2] = {sg, mate[sg]};
            if (!W.pair_blocks || W.pair_variant != ctx->opt_fp64_pair || W.pcn.n != (size_t)2 * S.n_steps)
                prepare_pair(ctx, W);
            std::vector<double> hcn2, hco2, pout(2 * kRed), pres;
            std::vector<int32_t> pit;
            for (int j = 0; j < 2; ++j) {
                schedule_row(S, seq ? seq[idx[j]] : 0, q[idx[j]], hcn, hco);
                hcn2.insert(hcn2.end(), hcn.begin(), hcn.end());
                hco2.insert(hco2.end(), hco.begin(), hco.end());
            }
            W.pcn.upload(hcn2.data(), hcn2.size(), s);
            W.pco.upload(hco2.data(), hco2.size(), s);
            pack_signal_fp64(ctx, W, gdir + 3 * sg, u0 ? d_u0.p : nullptr);
            stepper_ms_total += run_pair_fp64(ctx, W, u0 ? d_u0.p : nullptr, rtol, maxit, pit, pres, pout.data());
            k_pair_extract<<<(unsigned)((W.n_pad + 255) / 256), 256, 0, s>>>(
                W.n_pad, W.pu[S.n_steps % 3], W.saved.p + (size_t)idx[0] * W.n_pad,
                W.saved.p + (size_t)idx[1] * W.n_pad);
            BT_CUDA(cudaGetLastError());
            for (int j = 0; j < 2; ++j)
                record(idx[j], pout.data() + j * kRed, pit.data() + (size_t)j * S.n_steps,
                       pres.data() + (size_t)j * S.n_steps);
            if (st) st->kernel_launches += 5;
            continue;
        }
        schedule_row(S, seq ? seq[sg] : 0, q[sg], hcn, hco);
        W.cn.upload(hcn.data(), S.n_steps, s);
        W.co.upload(hco.data(), S.n_steps, s);
        if (ctx->per.on) {
            BT_REQUIRE(S.phase_set, BT_ERR_STATE, "pseudo-periodic boundaries need bt_set_schedule_phase");
            const double* Fo = S.F_old.data() + (size_t)(seq ? seq[sg] : 0) * S.n_steps;
            hps.resize(S.n_steps);
            for (int k = 0; k < S.n_steps; ++k) hps[k] = q[sg] * Fo[k];
            W.ps.upload(hps.data(), S.n_steps, s);
        }
        pack_signal_fp64(ctx, W, gdir + 3 * sg, u0 ? d_u0.p : nullptr);
        stepper_ms_total += run_steps_fp64(ctx, W, W.cn, W.co, S.n_steps, ctx->opt_fp64_extrapolate != 0, nullptr,
                                           nullptr, 1, rtol, maxit, &hit, &hres, hout.data());
        BT_CUDA(cudaMemcpyAsync(W.saved.p + (size_t)sg * W.n_pad, W.u[S.n_steps % 3].p,
                                W.n_pad * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        record(sg, hout.data(), hit.data(), hres.data());
        if (st) st->kernel_launches += 3;
    }
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    BT_CUDA(cudaEventSynchronize(ctx->ev2));
    float total_ms = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total_ms, ctx->ev0, ctx->ev2));
    if (st) {
        st->gpu_ms = total_ms;
        st->stepper_ms = stepper_ms_total;
    }
    ctx->last_nsig = nsig;
}

void get_solution_fp64(bt_ctx* ctx, int32_t index, double* u) {
    BT_REQUIRE(ctx->s64 && index >= 0 && index < ctx->s64->saved_nsig, BT_ERR_INVALID,
               "bt_get_solution: no such signal in the last FP64 solve");
    Solver64& W = *ctx->s64;
    BT_CUDA(cudaMemcpyAsync(u, W.saved.p + (size_t)index * W.n_pad, ctx->mesh.n_dofs * sizeof(double2),
                            cudaMemcpyDeviceToHost, ctx->stream));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
}

void free_solver64(bt_ctx* ctx) {
    delete ctx->s64;
    ctx->s64 = nullptr;
}

}  // namespace bt

namespace bt {

// ============================================================== adjoint ====
// Discrete adjoint of the FP64 Crank-Nicolson loop.
//
//   forward   A_n u_{n+1} = B_n u_n,   Sig = Re(w^T u_N)
//   adjoint   lambda_N = A_{N-1}^{-1} w,  lambda_n = A_{n-1}^{-1} B_n lambda_{n+1}
//   gradient  dSig/dxi = -Re sum_n lambda_{n+1}^T (dS/dxi) (theta u_{n+1} + (1-theta) u_n)
//
// A and B are complex symmetric, so the transposed solves are the same COCG
// steps run on a shifted schedule.  S = K + T + R is linear in every
// parameter: D_r (isotropic, per region), 1/T2_r and kappa of each region pair,
// so dS/dxi is the unit-coefficient element (or facet) matrix of the cells
// (facets) carrying xi; the contraction is done per cell / per interface facet
// and accumulated over steps on the device, then reduced once in index order.
// Forward states are recomputed from checkpoints every `stride` steps
// (default ceil(sqrt(N))).
namespace {

// acc6 (nullable): per cell, the contraction with the unit stiffness of each
// stored tensor component (xx, yy, zz, xy, xz, yz; an off-diagonal component
// sets both D_kl and D_lk), for gradients with respect to a per-cell D field.
__global__ void k_adj_cells(int64_t n_t, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                            const int32_t* __restrict__ comp, const int32_t* __restrict__ dof_of, int nc,
                            const double2* __restrict__ lam, const double2* __restrict__ un,
                            const double2* __restrict__ un1, double theta, double* __restrict__ accD,
                            double* __restrict__ accT, double* __restrict__ acc6) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_t) return;
    const int4 qv = reinterpret_cast<const int4*>(tets)[t];
    const int32_t v[4] = {qv.x, qv.y, qv.z, qv.w};
    double X[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) X[k][c] = xyz[(int64_t)v[k] * 3 + c];
    double E[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) E[r][c] = X[r + 1][c] - X[0][c];
    const double c00 = E[1][1] * E[2][2] - E[1][2] * E[2][1];
    const double c01 = E[1][2] * E[2][0] - E[1][0] * E[2][2];
    const double c02 = E[1][0] * E[2][1] - E[1][1] * E[2][0];
    const double det = E[0][0] * c00 + E[0][1] * c01 + E[0][2] * c02;
    const double id = 1.0 / det;
    double G[4][3];
    G[1][0] = c00 * id; G[1][1] = c01 * id; G[1][2] = c02 * id;
    G[2][0] = (E[0][2] * E[2][1] - E[0][1] * E[2][2]) * id;
    G[2][1] = (E[0][0] * E[2][2] - E[0][2] * E[2][0]) * id;
    G[2][2] = (E[0][1] * E[2][0] - E[0][0] * E[2][1]) * id;
    G[3][0] = (E[0][1] * E[1][2] - E[0][2] * E[1][1]) * id;
    G[3][1] = (E[0][2] * E[1][0] - E[0][0] * E[1][2]) * id;
    G[3][2] = (E[0][0] * E[1][1] - E[0][1] * E[1][0]) * id;
#pragma unroll
    for (int c = 0; c < 3; ++c) G[0][c] = -(G[1][c] + G[2][c] + G[3][c]);
    const double vol = fabs(det) / 6.0;
    const int f = comp[t];
    double2 L[4], V[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int32_t d = dof_of[(int64_t)v[k] * nc + f];
        L[k] = lam[d];
        const double2 a0 = un[d], a1 = un1[d];
        V[k] = make_double2(theta * a1.x + (1.0 - theta) * a0.x, theta * a1.y + (1.0 - theta) * a0.y);
    }
    // Re(L^T K V) and Re(L^T M V), unit coefficients
    double sK = 0.0, sM = 0.0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const double re = L[r].x * V[c].x - L[r].y * V[c].y;
            sK += vol * (G[r][0] * G[c][0] + G[r][1] * G[c][1] + G[r][2] * G[c][2]) * re;
            sM += (r == c ? vol / 10.0 : vol / 20.0) * re;
        }
    accD[t] -= sK;
    accT[t] -= sM;
    if (acc6) {
        // Re(L^T (grad phi_r)_k (grad phi_c)_l V) summed over r, c = (L^T G)_k . (G^T V)_l
        double lg[3][2], gv[3][2];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lg[k][0] = lg[k][1] = gv[k][0] = gv[k][1] = 0.0;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                lg[k][0] += G[r][k] * L[r].x;
                lg[k][1] += G[r][k] * L[r].y;
                gv[k][0] += G[r][k] * V[r].x;
                gv[k][1] += G[r][k] * V[r].y;
            }
        }
        auto re = [&](int k, int l) { return lg[k][0] * gv[l][0] - lg[k][1] * gv[l][1]; };
        double* o = acc6 + t * 6;
        o[0] -= vol * re(0, 0);
        o[1] -= vol * re(1, 1);
        o[2] -= vol * re(2, 2);
        o[3] -= vol * (re(0, 1) + re(1, 0));
        o[4] -= vol * (re(0, 2) + re(2, 0));
        o[5] -= vol * (re(1, 2) + re(2, 1));
    }
}

__global__ void k_adj_facets(int64_t n_if, const int32_t* __restrict__ fcell, const int32_t* __restrict__ fface,
                             const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                             const int32_t* __restrict__ nbr, const int32_t* __restrict__ comp,
                             const int32_t* __restrict__ dof_of, int nc, const double2* __restrict__ lam,
                             const double2* __restrict__ un, const double2* __restrict__ un1, double theta,
                             double* __restrict__ accK) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_if) return;
    const int32_t t = fcell[i];
    const int fa = fface[i];
    const int32_t nb = nbr[(int64_t)t * 4 + fa];
    const int f = comp[t], g = comp[nb];
    int32_t fv[3];
    int m = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k != fa) fv[m++] = tets[(int64_t)t * 4 + k];
    double P[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) P[k][c] = xyz[(int64_t)fv[k] * 3 + c];
    double e1[3], e2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        e1[c] = P[1][c] - P[0][c];
        e2[c] = P[2][c] - P[0][c];
    }
    const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                 cz = e1[0] * e2[1] - e1[1] * e2[0];
    const double area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
    double2 Lj[3], Vj[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int32_t da = dof_of[(int64_t)fv[k] * nc + f], db = dof_of[(int64_t)fv[k] * nc + g];
        const double2 la = lam[da], lb = lam[db];
        const double2 ua0 = un[da], ua1 = un1[da], ub0 = un[db], ub1 = un1[db];
        Lj[k] = make_double2(la.x - lb.x, la.y - lb.y);
        Vj[k] = make_double2(theta * (ua1.x - ub1.x) + (1.0 - theta) * (ua0.x - ub0.x),
                             theta * (ua1.y - ub1.y) + (1.0 - theta) * (ua0.y - ub0.y));
    }
    double sK = 0.0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            sK += (r == c ? area / 6.0 : area / 12.0) * (Lj[r].x * Vj[c].x - Lj[r].y * Vj[c].y);
    accK[i] -= sK;
}

}  // namespace

void adjoint_fp64(bt_ctx* ctx, double q, const double* gdir, int32_t seq, const double* u0, double rtol,
                  int32_t maxit, int32_t stride, double* sig, double* dD, double* dinvT2, double* dkappa,
                  bt_stats* st, double* dD_cell, double* dinvT2_cell) {
    Mesh& m = ctx->mesh;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    BT_REQUIRE(!(dD && ctx->coeffs.has_cell_D), BT_ERR_STATE,
               "bt_adjoint: per-region D gradients need per-region isotropic D (clear the per-cell tensor, or "
               "use bt_adjoint_cells)");
    BT_REQUIRE(!(dinvT2 && ctx->coeffs.has_cell_T2), BT_ERR_STATE,
               "bt_adjoint: per-region 1/T2 gradients need per-region 1/T2 (clear the per-cell T2, or use "
               "bt_adjoint_cells)");
    BT_REQUIRE(!ctx->per.on, BT_ERR_STATE,
               "bt_adjoint: not defined with pseudo-periodic boundaries (the mirror term is not transposed)");
    BT_REQUIRE(!ctx->coeffs.kappa_cr, BT_ERR_STATE,
               "bt_adjoint: gradients are defined for one permeability per facet (not the Crouzeix-Raviart mode)");
    if (!ctx->s64) ctx->s64 = new Solver64();
    Solver64& W = *ctx->s64;
    prepare_fp64(ctx, W);
    const int N = S.n_steps;
    const double th = S.theta;
    if (stride <= 0) stride = (int)std::ceil(std::sqrt((double)N));
    stride = std::max(1, std::min(stride, N));
    const int nck = (N + stride - 1) / stride;  // checkpoints u_0, u_stride, ...
    DevBuf<double> d_u0;
    if (u0) d_u0.upload(u0, m.n_v, s);
    std::vector<double> hcn, hco, hout(kRed);
    schedule_row(S, seq, q, hcn, hco);
    // adjoint schedule: step j builds lambda_{N-j} with A_{N-j-1} and B_{N-j}
    std::vector<double> acn(N), aco(N, 0.0);
    for (int j = 0; j < N; ++j) {
        acn[j] = hcn[N - 1 - j];
        if (j >= 1) aco[j] = hco[N - j];
    }
    DevBuf<double> d_cn, d_co, d_acn, d_aco;
    d_cn.upload(hcn.data(), N, s);
    d_co.upload(hco.data(), N, s);
    d_acn.upload(acn.data(), N, s);
    d_aco.upload(aco.data(), N, s);
    pack_signal_fp64(ctx, W, gdir, u0 ? d_u0.p : nullptr);
    const size_t vb = (size_t)W.n_pad * sizeof(double2);
    DevBuf<double2> ck, seg, lam;
    ck.alloc((size_t)(nck + 1) * W.n_pad);
    seg.alloc((size_t)(stride + 1) * W.n_pad);
    lam.alloc(W.n_pad);
    DevBuf<double> accD, accT, accK;
    accD.alloc(m.n_t);
    accD.zero(s);
    accT.alloc(m.n_t);
    accT.zero(s);
    DevBuf<double> acc6;
    if (dD_cell) {
        acc6.alloc((size_t)m.n_t * 6);
        acc6.zero(s);
    }
    accK.alloc(std::max<int64_t>(1, m.n_iface));
    accK.zero(s);
    std::vector<int32_t> hit;
    int64_t total_iters = 0;
    int32_t max_iters = 0;
    auto count = [&](const std::vector<int32_t>& v) {
        for (int32_t x : v) {
            total_iters += x;
            max_iters = std::max(max_iters, x);
        }
    };
    float ms = 0.0f;
    BT_CUDA(cudaEventRecord(ctx->ev0, s));
    // forward: checkpoints ck[0] = u_0, ck[j] = u_{j*stride}
    BT_CUDA(cudaMemcpyAsync(ck.p, W.u[0].p, vb, cudaMemcpyDeviceToDevice, s));
    ms += run_steps_fp64(ctx, W, d_cn, d_co, N, ctx->opt_fp64_extrapolate != 0, nullptr, ck.p + W.n_pad, stride,
                         rtol, maxit, &hit, nullptr, hout.data());
    count(hit);
    *sig = hout[0];
    // lambda_N = A_{N-1}^{-1} w  (x0 = 0)
    W.u[0].zero(s);
    W.u[2].zero(s);
    ms += run_steps_fp64(ctx, W, d_acn.p, d_aco.p, 1, false, W.w, nullptr, 1, rtol, maxit, &hit, nullptr,
                         nullptr);
    count(hit);
    BT_CUDA(cudaMemcpyAsync(lam.p, W.u[1].p, vb, cudaMemcpyDeviceToDevice, s));
    const unsigned cb = (unsigned)((m.n_t + 127) / 128), fb = (unsigned)((m.n_iface + 127) / 128);
    for (int sg = nck - 1; sg >= 0; --sg) {
        const int a0 = sg * stride, b0 = std::min(a0 + stride, N);
        // recompute u_{a0..b0} from the checkpoint (no extrapolation at the restart)
        BT_CUDA(cudaMemcpyAsync(seg.p, ck.p + (size_t)sg * W.n_pad, vb, cudaMemcpyDeviceToDevice, s));
        BT_CUDA(cudaMemcpyAsync(W.u[0].p, seg.p, vb, cudaMemcpyDeviceToDevice, s));
        BT_CUDA(cudaMemcpyAsync(W.u[2].p, seg.p, vb, cudaMemcpyDeviceToDevice, s));
        ms += run_steps_fp64(ctx, W, d_cn.p + a0, d_co.p + a0, b0 - a0, ctx->opt_fp64_extrapolate != 0, nullptr,
                             seg.p + W.n_pad, 1, rtol, maxit, &hit, nullptr, nullptr);
        count(hit);
        for (int n = b0 - 1; n >= a0; --n) {
            const double2* un = seg.p + (size_t)(n - a0) * W.n_pad;
            const double2* un1 = seg.p + (size_t)(n - a0 + 1) * W.n_pad;
            k_adj_cells<<<cb, 128, 0, s>>>(m.n_t, m.xyz, m.tets, m.comp, m.dof_of, m.n_comp, lam.p, un, un1, th,
                                           accD.p, accT.p, dD_cell ? acc6.p : nullptr);
            if (m.n_iface > 0)
                k_adj_facets<<<fb, 128, 0, s>>>(m.n_iface, m.iface_cell, m.iface_face, m.xyz, m.tets, m.nbr,
                                                m.comp, m.dof_of, m.n_comp, lam.p, un, un1, th, accK.p);
            BT_CUDA(cudaGetLastError());
            if (n >= 1) {  // lambda_n = A_{n-1}^{-1} B_n lambda_{n+1}
                const int j = N - n;
                BT_CUDA(cudaMemcpyAsync(W.u[0].p, lam.p, vb, cudaMemcpyDeviceToDevice, s));
                BT_CUDA(cudaMemcpyAsync(W.u[2].p, lam.p, vb, cudaMemcpyDeviceToDevice, s));
                ms += run_steps_fp64(ctx, W, d_acn.p + j, d_aco.p + j, 1, false, nullptr, nullptr, 1, rtol, maxit,
                                     &hit, nullptr, nullptr);
                count(hit);
                BT_CUDA(cudaMemcpyAsync(lam.p, W.u[1].p, vb, cudaMemcpyDeviceToDevice, s));
            }
        }
    }
    // reduce once, in index order
    std::vector<double> hD(m.n_t), hT(m.n_t), hK(m.n_iface);
    std::vector<int32_t> hreg(m.n_t), hfc(m.n_iface), hff(m.n_iface), hnb(m.n_t * 4);
    accD.download(hD.data(), m.n_t, s);
    accT.download(hT.data(), m.n_t, s);
    if (m.n_iface > 0) {
        accK.download(hK.data(), m.n_iface, s);
        m.iface_cell.download(hfc.data(), m.n_iface, s);
        m.iface_face.download(hff.data(), m.n_iface, s);
    }
    m.region.download(hreg.data(), m.n_t, s);
    m.nbr.download(hnb.data(), m.n_t * 4, s);
    if (dD_cell) acc6.download(dD_cell, (size_t)m.n_t * 6, s);
    if (dinvT2_cell) accT.download(dinvT2_cell, m.n_t, s);
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    BT_CUDA(cudaStreamSynchronize(s));
    const int nr = m.n_regions;
    for (int r = 0; r < nr; ++r) {
        if (dD) dD[r] = 0.0;
        if (dinvT2) dinvT2[r] = 0.0;
    }
    if (dkappa)
        for (int k = 0; k < nr * nr; ++k) dkappa[k] = 0.0;
    for (int64_t t = 0; t < m.n_t; ++t) {
        if (dD) dD[hreg[t]] += hD[t];
        if (dinvT2) dinvT2[hreg[t]] += hT[t];
    }
    if (dkappa) {
        std::vector<double> pair((size_t)nr * nr, 0.0);
        for (int64_t i = 0; i < m.n_iface; ++i) {
            const int32_t t = hfc[i];
            const int32_t nb = hnb[(size_t)t * 4 + hff[i]];
            const int r1 = std::min(hreg[t], hreg[nb]), r2 = std::max(hreg[t], hreg[nb]);
            pair[(size_t)r1 * nr + r2] += hK[i];
        }
        for (int r1 = 0; r1 < nr; ++r1)
            for (int r2 = r1; r2 < nr; ++r2) {
                dkappa[(size_t)r1 * nr + r2] = pair[(size_t)r1 * nr + r2];
                dkappa[(size_t)r2 * nr + r1] = pair[(size_t)r1 * nr + r2];
            }
    }
    float total = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total, ctx->ev0, ctx->ev2));
    if (st) {
        st->steps = N;
        st->max_iterations = max_iters;
        st->total_iterations = total_iters;
        st->max_rel_residual = rtol;
        st->refinements = 0;
        st->graph_launches = 0;
        st->kernel_launches = 0;
        st->gpu_ms = total;
        st->stepper_ms = ms;
    }
}

}  // namespace bt

namespace bt {

// extra[n][row] = -S_xi (theta u_{n+1} + (1-theta) u_n) for every step n: the
// forcing of the tangent-linear recursion (CSR rows = stepper rows).
__global__ void k_tl_forcing(int64_t n_dofs, int64_t n_pad, int32_t n_steps, const int32_t* __restrict__ row_ptr,
                             const int32_t* __restrict__ col, const double* __restrict__ sxi,
                             const double2* __restrict__ states, double theta, double2* __restrict__ extra) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n_steps * n_pad) return;
    const int64_t n = t / n_pad, i = t % n_pad;
    double2 y = make_double2(0.0, 0.0);
    if (i < n_dofs) {
        const double2* un = states + n * n_pad;
        const double2* u1 = states + (n + 1) * n_pad;
        for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
            const int c = col[e];
            const double s = sxi[e];
            y.x = fma(s, theta * u1[c].x + (1.0 - theta) * un[c].x, y.x);
            y.y = fma(s, theta * u1[c].y + (1.0 - theta) * un[c].y, y.y);
        }
    }
    extra[t] = make_double2(-y.x, -y.y);
}

// Tangent-linear FP64 run for one parameter xi (kind 0: D of region i, 1: 1/T2 of
// region i, 2: kappa of the region pair (i, j)):
//   A_n v_{n+1} = B_n v_n - (dS/dxi) (theta u_{n+1} + (1 - theta) u_n),   v_0 = 0,
// dSig/dxi = sum w Re(v_N).  dS/dxi is assembled with indicator coefficients into
// scratch matrices (the system's matrices and coefficients are untouched); the
// forward states are all kept on the device ((N+1) x n_pad complex values).
void tangent_fp64(bt_ctx* ctx, double q, const double* gdir, int32_t seq, const double* u0, int32_t kind, int32_t ri,
                  int32_t rj, double rtol, int32_t maxit, double* sig, double* dsig, bt_stats* st) {
    Mesh& m = ctx->mesh;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    BT_REQUIRE(!ctx->coeffs.has_cell_D && !ctx->coeffs.has_cell_T2, BT_ERR_STATE,
               "bt_tangent: derivatives are defined for per-region coefficients (clear per-cell D / T2)");
    BT_REQUIRE(!ctx->per.on, BT_ERR_STATE, "bt_tangent: not defined with pseudo-periodic boundaries");
    BT_REQUIRE(!ctx->coeffs.kappa_cr, BT_ERR_STATE,
               "bt_tangent: derivatives are defined for one permeability per facet (not the Crouzeix-Raviart mode)");
    const int nr = m.n_regions;
    BT_REQUIRE(kind >= 0 && kind <= 2 && ri >= 0 && ri < nr && (kind != 2 || (rj >= 0 && rj < nr && rj != ri)),
               BT_ERR_INVALID, "bt_tangent: bad parameter");
    // dS/dxi with indicator coefficients, into scratch matrices
    std::vector<double> eD(nr, 0.0), eT(nr, 0.0), eK((size_t)nr * nr, 0.0);
    if (kind == 0) eD[ri] = 1.0;
    if (kind == 1) eT[ri] = 1.0;
    if (kind == 2) eK[(size_t)ri * nr + rj] = eK[(size_t)rj * nr + ri] = 1.0;
    Coeffs ind;
    ind.D_region.upload(eD.data(), nr, s);
    ind.invT2_region.upload(eT.data(), nr, s);
    ind.kappa_pair.upload(eK.data(), (size_t)nr * nr, s);
    ind.set = true;
    Assembled scratch;
    std::swap(ctx->mat, scratch);
    std::swap(ctx->coeffs, ind);
    try {
        assemble_all(ctx);
    } catch (...) {
        std::swap(ctx->mat, scratch);
        std::swap(ctx->coeffs, ind);
        throw;
    }
    std::swap(ctx->mat, scratch);
    std::swap(ctx->coeffs, ind);
    const double* sxi = (kind == 0) ? scratch.K.p : (kind == 1) ? scratch.T.p : scratch.R.p;

    if (!ctx->s64) ctx->s64 = new Solver64();
    Solver64& W = *ctx->s64;
    prepare_fp64(ctx, W);
    const int N = S.n_steps;
    DevBuf<double> d_u0;
    if (u0) d_u0.upload(u0, m.n_v, s);
    std::vector<double> hcn, hco, hout(kRed);
    schedule_row(S, seq, q, hcn, hco);
    DevBuf<double> d_cn, d_co;
    d_cn.upload(hcn.data(), N, s);
    d_co.upload(hco.data(), N, s);
    pack_signal_fp64(ctx, W, gdir, u0 ? d_u0.p : nullptr);
    const size_t vb = (size_t)W.n_pad * sizeof(double2);
    DevBuf<double2> states, extra;
    states.alloc((size_t)(N + 1) * W.n_pad);
    extra.alloc((size_t)N * W.n_pad);
    std::vector<int32_t> hit1, hit2;
    BT_CUDA(cudaEventRecord(ctx->ev0, s));
    BT_CUDA(cudaMemcpyAsync(states.p, W.u[0].p, vb, cudaMemcpyDeviceToDevice, s));
    float ms = run_steps_fp64(ctx, W, d_cn, d_co, N, ctx->opt_fp64_extrapolate != 0, nullptr, states.p + W.n_pad, 1,
                              rtol, maxit, &hit1, nullptr, hout.data());
    *sig = hout[0];
    const int64_t total = (int64_t)N * W.n_pad;
    k_tl_forcing<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(m.n_dofs, W.n_pad, N, m.row_ptr, m.col, sxi,
                                                                  states.p, S.theta, extra.p);
    BT_CUDA(cudaGetLastError());
    // v_0 = 0 (also the extrapolation's previous level)
    for (int k = 0; k < 3; ++k) BT_CUDA(cudaMemsetAsync(W.u[k].p, 0, vb, s));
    ms += run_steps_fp64(ctx, W, d_cn, d_co, N, ctx->opt_fp64_extrapolate != 0, nullptr, nullptr, 1, rtol, maxit,
                         &hit2, nullptr, hout.data(), extra.p);
    *dsig = hout[0];
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    BT_CUDA(cudaEventSynchronize(ctx->ev2));
    if (st) {
        st->steps = N;
        st->max_iterations = 0;
        st->total_iterations = 0;
        for (int32_t x : hit1) {
            st->total_iterations += x;
            st->max_iterations = std::max(st->max_iterations, x);
        }
        for (int32_t x : hit2) {
            st->total_iterations += x;
            st->max_iterations = std::max(st->max_iterations, x);
        }
        st->max_rel_residual = rtol;
        st->refinements = 0;
        st->graph_launches = 0;
        st->kernel_launches = 3;
        st->stepper_ms = ms;
        float total_ms = 0.0f;
        BT_CUDA(cudaEventElapsedTime(&total_ms, ctx->ev0, ctx->ev2));
        st->gpu_ms = total_ms;
    }
}

}  // namespace bt
