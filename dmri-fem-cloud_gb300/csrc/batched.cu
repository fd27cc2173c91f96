// Batched mixed-precision Crank-Nicolson stepper: up to 512 signals (gradient
// directions, b-values, sequences) of one mesh advance together in one
// persistent cooperative launch, as a multi-RHS SpMM over the shared CSR
// matrices A_re = M/k + theta (K + T + R), Jx, Jy, Jz.
//
// Precision.  GB300 runs FP64 at a small fraction of its FP32 rate, so no
// FP64 arithmetic is used per matrix entry.  Each time step solves the
// correction form of the reference's step (DmriFemLib.py:901-907):
//     A_n d = r,   r = b_n - A_n u  =  -(S u + i (cn + co) J_g u)   at u = u_n
// where S = K + T + R and J_g = sum_k g_k J_k (theta-general: B - A = -S).
// * u is kept as a double-float pair (hi + lo, FP32 each, ~44 bits), and the
//   outer residual r is formed with error-free FP32 transformations (TwoProd by
//   FMA, TwoSum) against double-float matrix values, so it is as accurate as
//   an FP64 SpMV;
// * the correction d is found by Jacobi-COCG entirely in FP32 (vectors and
//   matrix hi parts), to a relative tolerance of 3e-6 in the first sweep.  The
//   gradient winds the phase of u across the mesh, so COCG's unconjugated forms
//   r^T z and p^T A p cancel by orders of magnitude for a complex right-hand
//   side and FP32 COCG then stalls.  Each signal's correction is therefore
//   solved as two right-hand sides, Re(r) and Im(r) (d = d_re + i d_im), whose
//   Krylov vectors stay nearly real (the imaginary part of A is a few percent
//   of its real part), and the lane-local sums are compensated (Kahan) and
//   combined in FP64;
// * the outer residual is updated in double-float, r -= A d, u += d, and
//   further FP32 sweeps (tolerance 1e-2) run until ||r|| <= rtol ||b||, with
//   ||b|| estimated as ||(1/k) w o u|| (w = lumped mass).
// The signal int Re(u) is accumulated in FP64 at the end.
//
// Layout.  Inner vectors are [row][Rp] complex FP32 "slots" (slots 2s, 2s+1
// are Re / Im of signal s; Rp a multiple of the chunk size C), so the gather of
// a neighbour row reads C consecutive complex values: a warp-unit of LPR lanes
// per row x (32/LPR) rows, each lane holding the 2 slots of one signal (one
// 16-byte load per neighbour).  u and the outer residual are [row][Rp/2]
// double-float complex per signal.  Matrix entries are loaded
// once per unit and broadcast.  LPR ("lanes per row") and the blocks per SM
// are chosen by a measuring autotuner (autotune_mixed).
//
// Reductions are deterministic: lanes sum their rows in order, warps combine
// row slots by XOR shuffles, blocks combine warps of the same RHS chunk in
// warp order, and the grid sums block partials in block order (in one stage
// when the partials are few, otherwise in two stages with an extra barrier).
#include "bt_common.cuh"

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>

namespace bt {

constexpr int kWarpsB = 8;
constexpr int kThreadsB = kWarpsB * 32;
constexpr int kMaxRhs = 512;
constexpr int kNV = 4;  // values per RHS in one reduction
constexpr int kNV1 = 9; // values per RHS in the reduction of the single-reduction COCG iteration

struct MixArgs;

struct SolverMixed {
    int64_t n = 0;
    int32_t Rp = 0;
    int32_t nb = 0;
    DevBuf<float4> mA, mL;    // per nnz: {A,Jx,Jy,Jz} hi and lo
    DevBuf<float2> mS;        // per nnz: S hi, lo
    DevBuf<float4> dg;        // per row: diagonal {A,Jx,Jy,Jz} (hi)
    DevBuf<double> w;         // per row signal weight
    DevBuf<int32_t> rcomp;
    DevBuf<float2> uh, ul, rh, rl, d0, d1, ri, z, p, q;  // [n][Rp]
    DevBuf<float2> z1, w1, q1;   // [n][Rp]: second buffers of the single-reduction iteration
    DevBuf<float2> hc, t1, t2, t3, ex;   // per signal [n][Rp/2]: extrapolated guess (MixArgs)
    DevBuf<float2> partials, fin;   // double-float (hi, lo) sums
    DevBuf<double> sigpart;      // [warps][64][1+kMaxCompartments]
    DevBuf<unsigned> bar;
    DevBuf<int> status;
    DevBuf<double> fnew, fold;   // [n_seq][n_steps]
    DevBuf<double> Fint;         // [n_seq][n_steps]: F(tp), pseudo-periodic phase
    DevBuf<double> gvd;          // [Rp][3] gradient directions in FP64 (pseudo-periodic phase)
    DevBuf<double> qv;           // [Rp]
    DevBuf<float> gv;            // [Rp][3]
    DevBuf<int32_t> seqv;        // [Rp]
    DevBuf<double> sig;          // [Rp][1 + kMaxCompartments]
    DevBuf<int32_t> iters, sweeps;  // [n_steps]
    DevBuf<float> diag;
    DevBuf<double> u0;
    // final solutions of the last solve: [nsig][n] complex (hi + lo, as double2)
    std::vector<double2> saved;
    int32_t saved_nsig = 0;
    struct Geo {
        int lpr, per_sm, blocked;
    };
    std::map<std::pair<int64_t, int32_t>, Geo> tuned;  // (n, R) -> launch geometry
    DevBuf<MixArgs> margs;   // several meshes in one launch (kept by the first mesh's context)
    DevBuf<int> mfirst;
    std::map<std::vector<int64_t>, int> tuned_multi;   // (n_dofs, R per mesh) -> lanes per row
};

struct MixArgs {
    int32_t n;
    int32_t Rp;
    int32_t R;            // real RHS (the rest is padding)
    const int32_t* __restrict__ row_ptr;
    const int32_t* __restrict__ col;
    const float4* __restrict__ mA;
    const float4* __restrict__ mL;
    const float2* __restrict__ mS;
    const float4* __restrict__ dg;
    const double* __restrict__ w;
    const int32_t* __restrict__ rcomp;
    float2* uh;  // per signal: [row][Rp/2] complex (double-float hi / lo)
    float2* ul;
    float2* rh;
    float2* rl;
    float4* dv[2];
    float4* ri;
    float4* z;
    float4* p;
    float4* q;
    // second buffers of the single-reduction iteration (z, w~, q~ alternate between
    // even and odd iterations: buffer 0 is z / ri / q, buffer 1 these)
    float4* z1;
    float4* w1;
    float4* q1;
    // extrapolated initial guess of order extrap (0 u_n, 1 linear ... 4): per signal,
    // hc = this step's total correction u_{n+1} - u_n (the offset e after phase S),
    // t1..t3 = backward differences of u at u_n (d_n, d_n - d_{n-1}, ...; own rows
    // only) and ex = the next step's offset (gathered by phase S)
    float2* hc;
    float2* t1;
    float2* t2;
    float2* t3;
    float2* ex;
    int32_t extrap;
    float2* partials;
    float2* fin;
    double* sigpart;
    unsigned* bar;
    int* status;
    const double* __restrict__ fnew;
    const double* __restrict__ fold;
    const double* __restrict__ qv;
    const float* __restrict__ gv;
    const int32_t* __restrict__ seqv;
    int32_t n_steps;
    int32_t sched_stride;  // steps per schedule row (n_steps may be fewer when tuning)
    int32_t maxit;
    int32_t max_sweeps;
    float theta;
    float inv_k;
    float rtol;
    float eps_first;
    float eps_next;
    int32_t reduce_mode;  // grid sums: 0 the last block to arrive, 1 every block, 2 two stages (see grid_reduce)
    int32_t blocked;      // rows: 0 interleaved over all warps, 1 contiguous range per block
    int32_t* iters;
    int32_t* sweeps;
    double* sig;  // [Rp][1+kMaxCompartments]
    float* diag;  // failure report: kind, step, sweep, iteration, worst rr2/target, RHS
    // pseudo-periodic boundary term of the right-hand side (nullable per_ptr),
    // evaluated in FP64 in phase S: (1 - theta) sum_e val.c e^{i q F(tp) g.(x,y,z)} u_n[col]
    const int32_t* __restrict__ per_ptr;
    const int32_t* __restrict__ per_col;
    const PerVal* __restrict__ per_val;
    const double* __restrict__ Fint;
    const double* __restrict__ gvd;
    double theta_d;
    // discrete adjoint (adjoint_mixed): the first step's right-hand side is the
    // signal weight w (from a zero state), and the state after every save_every-th
    // step is copied to save_h / save_l [(step + 1) / save_every - 1][n][Rp/2]
    float growth2;        // a slot ends its sweep when rr2 > growth2 * (smallest rr2 of the sweep)
    int32_t rhs_w;
    int32_t save_every;
    float2* save_h;
    float2* save_l;
    unsigned long long wait_ns;  // time limit of every grid-wide wait
    int32_t stall;               // failure-detection hook: the first wait runs out (stalled_wait on bar[4])
};

// ------------------------------------------------------------ double-float ----
struct DF {
    float h, l;
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// acc += (ah + al) * (xh + xl), error-free product of the hi parts
__device__ __forceinline__ void df_fma(DF& acc, float ah, float al, float xh, float xl) {
    const float p = ah * xh;
    float e = fmaf(ah, xh, -p);
    e = fmaf(ah, xl, e);
    e = fmaf(al, xh, e);
    float s, t;
    two_sum(acc.h, p, s, t);
    acc.h = s;
    acc.l += t + e;
}
__device__ __forceinline__ DF df_norm(DF a) {
    DF r;
    r.h = a.h + a.l;
    r.l = a.l - (r.h - a.h);
    return r;
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    float s, e;
    two_sum(a.h, b.h, s, e);
    e += a.l + b.l;
    DF r;
    r.h = s + e;
    r.l = e - (r.h - s);
    return r;
}
__device__ __forceinline__ DF df_scale(DF a, float c) {
    const float p = a.h * c;
    const float e = fmaf(a.h, c, -p);
    DF r;
    r.h = p;
    r.l = fmaf(a.l, c, e);
    return df_norm(r);
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// Smith's complex division: no squared magnitudes, so FP32 COCG scalars that
// are themselves sums of squared residuals (~1e-25) neither underflow nor
// overflow here.
__device__ __forceinline__ float2 cdivf(float2 a, float2 b) {
    if (fabsf(b.x) >= fabsf(b.y)) {
        const float r = b.y / b.x, d = fmaf(b.y, r, b.x);
        return make_float2(fmaf(a.y, r, a.x) / d, fmaf(-a.x, r, a.y) / d);
    }
    const float r = b.x / b.y, d = fmaf(b.x, r, b.y);
    return make_float2(fmaf(a.x, r, a.y) / d, fmaf(a.y, r, -a.x) / d);
}
__device__ __forceinline__ float2 cinvf(float2 b) { return cdivf(make_float2(1.0f, 0.0f), b); }
__device__ __forceinline__ bool cnonzero(float2 v) {
    return (v.x != 0.0f || v.y != 0.0f) && isfinite(v.x) && isfinite(v.y);
}
// Compensated (Kahan) FP32 accumulator.  The COCG scalars are sums of
// products that cancel strongly, and plain FP32 sequential sums then lose the
// step length and COCG stalls.  Lanes accumulate compensated, and every
// combination above the lane is done in double-float (reduce_rhs).
struct KF {
    float s, c;
};
__device__ __forceinline__ void kadd(KF& a, float x) {
    const float y = x - a.c;
    const float t = a.s + y;
    a.c = (t - a.s) - y;
    a.s = t;
}

// -------------------------------------------------------------- reductions ----
// Each lane holds compensated sums v[2][NV] for its two slots.  Lane sums are
// combined as double-float pairs (error-free TwoSum), never in FP64, which is
// slow on this GPU.  On return out[][] holds the grid-wide sums as double-float
// (hi, lo) pairs, bitwise identical in every block.
__device__ __forceinline__ float2 dfa(float2 a, float2 b) {  // (hi, lo) + (hi, lo)
    float s, e;
    two_sum(a.x, b.x, s, e);
    e += a.y + b.y;
    const float h = s + e;
    return make_float2(h, e - (h - s));
}

template <int LPR, int NV>
__device__ __forceinline__ bool reduce_rhs(KF (&v)[2][NV], float2 (&out)[2][NV], const MixArgs& a, int chunk,
                                           int r0, unsigned nb, unsigned bid, unsigned& gen, float2* smem) {
    constexpr int C = 2 * LPR;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float2 d[2][NV];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const float h = v[j][k].s - v[j][k].c;   // Kahan: true sum = s - c
            d[j][k] = make_float2(h, (v[j][k].s - h) - v[j][k].c);
        }
    // combine the row slots of the warp
#pragma unroll
    for (int o = 16; o >= LPR; o >>= 1) {
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const float2 t = make_float2(__shfl_xor_sync(0xffffffffu, d[j][k].x, o),
                                             __shfl_xor_sync(0xffffffffu, d[j][k].y, o));
                d[j][k] = dfa(d[j][k], t);
            }
    }
    if (lane < LPR) {
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < NV; ++k) smem[(wib * C + lane * 2 + j) * NV + k] = d[j][k];
    }
    __syncthreads();
    const int nchunks = a.Rp / C;
    // block partial for every slot: sum over this block's warps of that chunk, in order
    for (int t = threadIdx.x; t < a.Rp * NV; t += blockDim.x) {
        const int r = t / NV, k = t % NV;
        const int c = r / C, o = r % C;
        float2 s = make_float2(0.f, 0.f);
        for (int wb = 0; wb < kWarpsB; ++wb)
            if ((int)((bid * kWarpsB + wb) % nchunks) == c) s = dfa(s, smem[(wb * C + o) * NV + k]);
        a.partials[(size_t)bid * a.Rp * NV + t] = s;
    }
    const int V = a.Rp * NV;
    if (a.reduce_mode == 1) {
        // every block sums all partials itself, in the same fixed order as the last
        // block of mode 0 (so the sums are bitwise those of mode 0): no block waits
        // for another block's sums.  The blocks arrive on a 64-bit counter that only
        // grows; arrivals of consecutive reductions cannot interleave (a block
        // arrives for the next one only after all have arrived for this one), so a
        // block's own ticket tells it how many arrivals end this reduction.
        __shared__ int s_ok1;
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long* ctr = reinterpret_cast<unsigned long long*>(a.bar + 2);
            const unsigned long long ticket = atom_add_acqrel_u64(ctr, 1ull);
            const unsigned long long want = (ticket / nb + 1ull) * nb;
            int ok = 1;
            if (ticket + 1ull != want) {
                const unsigned long long t0 = globaltimer_ns();
                unsigned spins = 0;
                while (ld_acquire_u64(ctr) < want) {
                    if (++spins > kBarrierMaxSpins || (spins & 255u) == 0u &&
                        (globaltimer_ns() - t0 > a.wait_ns || ld_relaxed_i32(a.status) != DEV_OK)) {
                        atomicCAS(a.status, DEV_OK, DEV_TIMEOUT);
                        ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            s_ok1 = ok;
        }
        __syncthreads();
        if (!s_ok1) return false;
        int G = 32;
        while (G > 1 && V * G > (int)blockDim.x) G >>= 1;
        const int part = threadIdx.x % G;
        for (int t0 = 0; t0 < V; t0 += blockDim.x / G) {
            const int t = t0 + threadIdx.x / G;
            float2 s = make_float2(0.f, 0.f);
            if (t < V)
                for (unsigned b0 = part; b0 < nb; b0 += 8u * G) {
                    float2 tv[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const unsigned b = b0 + (unsigned)G * u;
                        tv[u] = (b < nb) ? __ldcg(&a.partials[(size_t)b * V + t]) : make_float2(0.f, 0.f);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) s = dfa(s, tv[u]);
                }
            for (int o = G / 2; o > 0; o >>= 1)
                s = dfa(s, make_float2(__shfl_xor_sync(0xffffffffu, s.x, o), __shfl_xor_sync(0xffffffffu, s.y, o)));
            if (part == 0 && t < V) smem[t] = s;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < NV; ++k) out[j][k] = smem[(r0 + j) * NV + k];
    } else if (a.reduce_mode == 2) {
        if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return false;
        // stage 2: one warp per value; lane l adds blocks l, l+32, ... and the
        // warp combines the 32 lane sums in a fixed butterfly (lane 0's order)
        const int gw = bid * kWarpsB + wib;
        for (int t = gw; t < V; t += nb * kWarpsB) {
            float2 s = make_float2(0.f, 0.f);
            for (unsigned b0 = lane; b0 < nb; b0 += 4u * 32u) {
                float2 tv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const unsigned b = b0 + 32u * u;
                    tv[u] = (b < nb) ? __ldcg(&a.partials[(size_t)b * V + t]) : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) s = dfa(s, tv[u]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                s = dfa(s, make_float2(__shfl_xor_sync(0xffffffffu, s.x, o), __shfl_xor_sync(0xffffffffu, s.y, o)));
            if (lane == 0) a.fin[t] = s;
        }
        if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return false;
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                out[j][k] = __ldcg(&a.fin[(r0 + j) * NV + k]);
            }
    } else {
        // one stage: the last block to arrive sums all partials (G lanes per value
        // stride over the blocks and combine in a fixed butterfly, so the sums do not
        // depend on which block is last), publishes them in fin and releases the
        // others, which read only the V sums
        __shared__ int s_last, s_ok;
        const unsigned target = gen + 1;
        // every thread makes its own stores (this phase's vectors and the partials)
        // visible device-wide before the block arrives: the arrival is one thread's
        // release, and we do not rely on it covering the other warps' stores
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            // no status check before arriving (it would cost a round trip): a block
            // that left on an error never arrives, and the waiters below see the
            // status within 256 polls
            s_ok = 1;
            s_last = (atom_add_acqrel_u32(&a.bar[0], 1u) == nb - 1);
        }
        __syncthreads();
        if (s_last) {
            int G = 32;
            while (G > 1 && V * G > (int)blockDim.x) G >>= 1;
            const int part = threadIdx.x % G;
            for (int t0 = 0; t0 < V; t0 += blockDim.x / G) {
                const int t = t0 + threadIdx.x / G;
                float2 s = make_float2(0.f, 0.f);
                if (t < V)
                    for (unsigned b0 = part; b0 < nb; b0 += 8u * G) {
                        float2 tv[8];   // eight independent loads in flight; zero padding adds exactly nothing
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const unsigned b = b0 + (unsigned)G * u;
                            tv[u] = (b < nb) ? __ldcg(&a.partials[(size_t)b * V + t]) : make_float2(0.f, 0.f);
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) s = dfa(s, tv[u]);
                    }
                for (int o = G / 2; o > 0; o >>= 1)
                    s = dfa(s, make_float2(__shfl_xor_sync(0xffffffffu, s.x, o), __shfl_xor_sync(0xffffffffu, s.y, o)));
                if (part == 0 && t < V) {
                    smem[t] = s;
                    __stcg(&a.fin[t], s);
                    __threadfence();
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                a.bar[0] = 0;
                st_release_u32(&a.bar[1], target);
            }
        } else {
            if (threadIdx.x == 0) {
                const unsigned long long t0 = globaltimer_ns();
                unsigned spins = 0;
                while (ld_acquire_u32(&a.bar[1]) != target) {
                    if (++spins > kBarrierMaxSpins || (spins & 255u) == 0u &&
                        (globaltimer_ns() - t0 > a.wait_ns || ld_relaxed_i32(a.status) != DEV_OK)) {
                        atomicCAS(a.status, DEV_OK, DEV_TIMEOUT);
                        s_ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            __syncthreads();
            if (!s_ok) return false;
            for (int t = threadIdx.x; t < V; t += blockDim.x) smem[t] = __ldcg(&a.fin[t]);
        }
        gen = target;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < NV; ++k) out[j][k] = smem[(r0 + j) * NV + k];
    }
    __syncthreads();
    return true;
}

// (1 - theta) sum_e c_e exp(i ps g.shift_e) u_n[col_e] of one boundary row, in
// FP64.  Kept out of line: its sincos (with the local array of the large-
// argument reduction) would otherwise weigh on the register allocation of the
// whole persistent kernel.
__device__ __noinline__ double2 periodic_term(const MixArgs& a, int row, int r0, int c4, int Rp4, double ps) {
    const double g0 = a.gvd[r0 * 3 + 0], g1 = a.gvd[r0 * 3 + 1], g2 = a.gvd[r0 * 3 + 2];
    double bx = 0.0, by = 0.0;
    for (int32_t e = a.per_ptr[row]; e < a.per_ptr[row + 1]; ++e) {
        const PerVal v = a.per_val[e];
        double sn, cs;
        sincos(ps * (g0 * v.x + g1 * v.y + g2 * v.z), &sn, &cs);
        const size_t ki = (size_t)a.per_col[e] * Rp4 + c4;
        const float2 kh = a.uh[ki], kl = a.ul[ki];
        const double ux = (double)kh.x + (double)kl.x, uy = (double)kh.y + (double)kl.y;
        bx = fma(v.c, cs * ux - sn * uy, bx);
        by = fma(v.c, sn * ux + cs * uy, by);
    }
    return make_double2((1.0 - a.theta_d) * bx, (1.0 - a.theta_d) * by);
}

// ------------------------------------------------- single-reduction COCG ----
// The lane's two slots of a float4 are (x, y) and (z, w).
__device__ __forceinline__ float2 slot_of(const float4 v, const int j) {
    return j ? make_float2(v.z, v.w) : make_float2(v.x, v.y);
}
__device__ __forceinline__ double2 dd2(const float2 hi, const float2 lo) {   // two double-float sums -> complex
    return make_double2((double)hi.x + (double)hi.y, (double)lo.x + (double)lo.y);
}

// q~_{k-1} = w~_{k-1} + beta_{k-1} q~_{k-2} and z_k = z_{k-1} - alpha_{k-1} q~_{k-1} for
// the lane's two slots.  Every row that gathers z_k of a neighbour forms it with
// this function from the same stored values, and so does the neighbour's owner:
// all of them get the same bits.
__device__ __forceinline__ float4 next_z(const float4 z, const float4 w, const float4 q, const float2 (&al)[2],
                                          const float2 (&be)[2], float4& qn) {
    qn.x = fmaf(be[0].x, q.x, fmaf(-be[0].y, q.y, w.x));
    qn.y = fmaf(be[0].x, q.y, fmaf(be[0].y, q.x, w.y));
    qn.z = fmaf(be[1].x, q.z, fmaf(-be[1].y, q.w, w.z));
    qn.w = fmaf(be[1].x, q.w, fmaf(be[1].y, q.z, w.w));
    float4 zn;
    zn.x = fmaf(-al[0].x, qn.x, fmaf(al[0].y, qn.y, z.x));
    zn.y = fmaf(-al[0].x, qn.y, fmaf(-al[0].y, qn.x, z.y));
    zn.z = fmaf(-al[1].x, qn.z, fmaf(al[1].y, qn.w, z.z));
    zn.w = fmaf(-al[1].x, qn.w, fmaf(-al[1].y, qn.z, z.w));
    return zn;
}

// Inner FP32 Jacobi-COCG with ONE grid-wide reduction per iteration.
//
// With D the Jacobi diagonal, the iteration keeps the scaled residual z = D^-1 r,
// w~ = D^-1 A z, q~ = D^-1 q (q = A p), p and the correction d.  Iteration k
// (k = 0, 1, ...; alpha_{k-1}, beta_{k-1} known, both 0 for k = 0) does, in one
// pass over the rows:
//     q~_{k-1} = w~_{k-1} + beta_{k-1} q~_{k-2}      (also for every neighbour)
//     z_k      = z_{k-1} - alpha_{k-1} q~_{k-1}      (also for every neighbour)
//     w_k      = A z_k                               (the SpMV)
//     p_{k-1}  = z_{k-1} + beta_{k-1} p_{k-2},  d_k = d_{k-1} + alpha_{k-1} p_{k-1}
// and the lane sums of rho_k = r_k^T z_k, |r_k|^2, delta_k = z_k^T w_k,
// sigma_k = z_k^T q_{k-1} and mu_{k-1} = p_{k-1}^T q_{k-1} (r = D z, q = D q~).
// Neighbours' z_k are formed from their stored z_{k-1}, w~_{k-1}, q~_{k-2} (the
// three gathered vectors alternate between two buffers, so nobody overwrites
// what another row still reads), hence no barrier is needed between the update
// and the SpMV.  After the one reduction:
//     beta_k = rho_k / rho_{k-1},
//     mu_k   = p_k^T A p_k = delta_k + 2 beta_k sigma_k + beta_k^2 mu_{k-1}
// (only A = A^T and q_{k-1} = A p_{k-1} are used, with mu_{k-1} summed directly,
// so no recurrence error accumulates in mu), alpha_k = rho_k / mu_k; the scalars
// are combined in FP64.  This is the Chronopoulos-Gear rearrangement of CG
// (Chronopoulos & Gear, J. Comput. Appl. Math. 25, 1989) applied to COCG's
// unconjugated forms, with the Jacobi scaling folded into the stored vectors.
// Vector traffic per slot and iteration: z, w~, q~ (gathered), p, d read; z, w~,
// q~, p, d written -- ten accesses, against twelve and two reductions for the
// two-reduction form.  Activity, divergence and stagnation rules are the same.
// Returns false when a reduction failed (the kernel must leave).
template <int LPR>
__device__ __forceinline__ bool inner_single(const MixArgs& a, MixArgs& b, const float eps, float (&rr2)[2],
                                             const float (&rrs)[2], const float (&tolb2)[2], float (&rrmin)[2],
                                             float (&rrmark)[2], int (&itmark)[2], bool (&act)[2], int& it,
                                             bool& failed, const int step, const int sweep, const float (&cn)[2],
                                             const float (&gx)[2], const float (&gy)[2], const float (&gz)[2],
                                             const int dsel, const int g0, const int gend, const int gstride,
                                             const int slot, const int r0, const int c4, const int Rp4,
                                             const int chunk, const unsigned nb, const unsigned bid, unsigned& gen,
                                             unsigned& flip, float2* const part0, float2* const part1,
                                             float2* smem) {
    constexpr int G = 32 / LPR;
    constexpr bool kShared = (LPR >= 8);
    const int lane = threadIdx.x & 31;
    float2 al[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    float2 be[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    double2 rho_p[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    float4* const P = a.p;
    float4* const Dv = a.dv[dsel];
    const float4 f4z = make_float4(0.f, 0.f, 0.f, 0.f);
    while (true) {
#pragma unroll
        for (int j = 0; j < 2; ++j)
            act[j] = (r0 + j < a.R) && rr2[j] > eps * eps * rrs[j] && rr2[j] > 0.09f * tolb2[j] &&
                     rr2[j] <= a.growth2 * rrmin[j] && it - itmark[j] < 64;
        if (!__syncthreads_or(act[0] || act[1])) break;
        if (it >= a.maxit) {
            if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
#pragma unroll
            for (int j = 0; j < 2; ++j)
                if (bid == 0 && act[j]) {
                    a.diag[0] = 1.0f; a.diag[1] = (float)step; a.diag[2] = (float)sweep; a.diag[3] = (float)it;
                    a.diag[4] = rr2[j] / fmaxf(eps * eps * rrs[j], 1e-38f);
                    a.diag[5] = (float)(r0 / 2);
                }
            failed = true;
            break;
        }
#pragma unroll
        for (int j = 0; j < 2; ++j)
            if (!act[j]) al[j] = be[j] = make_float2(0.f, 0.f);   // a finished slot keeps its d
        // even iterations read buffer 0 and write buffer 1, odd ones the reverse
        const bool odd = (it & 1) != 0;
        const float4* const Zr = odd ? a.z1 : a.z;
        const float4* const Wr = odd ? a.w1 : a.ri;
        const float4* const Qr = odd ? a.q1 : a.q;
        float4* const Zw = odd ? a.z : a.z1;
        float4* const Ww = odd ? a.ri : a.w1;
        float4* const Qw = odd ? a.q : a.q1;
        KF v[2][kNV1];
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < kNV1; ++k) v[j][k] = KF{0.0f, 0.0f};
        const bool lane_active = act[0] || act[1];
        for (int g = (kShared || lane_active) ? g0 : gend; g < gend; g += gstride) {
            const int row_raw = g * G + slot;
            if (!kShared && row_raw >= a.n) continue;
            const bool row_ok = row_raw < a.n;
            const int row = row_ok ? row_raw : a.n - 1;
            const bool mine = row_ok && lane_active;
            float2 sA[2], sx[2], sy[2], sz[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) sA[j] = sx[j] = sy[j] = sz[j] = make_float2(0.f, 0.f);
            const int e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
            auto acc_entry = [&](const float4 m, const float4 zz) {
                const float2 zj[2] = {make_float2(zz.x, zz.y), make_float2(zz.z, zz.w)};
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    sA[j].x = fmaf(m.x, zj[j].x, sA[j].x); sA[j].y = fmaf(m.x, zj[j].y, sA[j].y);
                    sx[j].x = fmaf(m.y, zj[j].x, sx[j].x); sx[j].y = fmaf(m.y, zj[j].y, sx[j].y);
                    sy[j].x = fmaf(m.z, zj[j].x, sy[j].x); sy[j].y = fmaf(m.z, zj[j].y, sy[j].y);
                    sz[j].x = fmaf(m.w, zj[j].x, sz[j].x); sz[j].y = fmaf(m.w, zj[j].y, sz[j].y);
                }
            };
            if constexpr (kShared) {
                // windows of 4 entries: lane gl < 4 of the row's group loads entry gl, the
                // group shares column and values by shuffles, then 4 x 3 gathers go out
                constexpr int W = 4;
                const int gl = lane % LPR;
                const int nn = e1 - e0;
                const int nmax = __reduce_max_sync(0xffffffffu, nn);
                for (int off = 0; off < nmax; off += W) {
                    const bool ok = gl < W && off + gl < nn;
                    const int my_c = ok ? a.col[e0 + off + gl] : row;
                    const float4 my_m = ok ? a.mA[e0 + off + gl] : f4z;
                    float4 zz[W], ww[W], qq[W];
#pragma unroll
                    for (int u = 0; u < W; ++u) {
                        const int c = __shfl_sync(0xffffffffu, my_c, u, LPR);
                        const size_t ni = (size_t)c * Rp4 + c4;
                        zz[u] = mine ? Zr[ni] : f4z;
                        ww[u] = mine ? Wr[ni] : f4z;
                        qq[u] = mine ? Qr[ni] : f4z;
                    }
#pragma unroll
                    for (int u = 0; u < W; ++u) {
                        float4 m;
                        m.x = __shfl_sync(0xffffffffu, my_m.x, u, LPR);
                        m.y = __shfl_sync(0xffffffffu, my_m.y, u, LPR);
                        m.z = __shfl_sync(0xffffffffu, my_m.z, u, LPR);
                        m.w = __shfl_sync(0xffffffffu, my_m.w, u, LPR);
                        float4 qn;
                        acc_entry(m, next_z(zz[u], ww[u], qq[u], al, be, qn));
                    }
                }
            } else {
                // four neighbours (twelve gathers) in flight per lane; the tail of a
                // row is predicated (a missing entry reads the own row times zero)
                for (int e = e0; e < e1; e += 4) {
                    int cc[4];
                    float4 mm[4], zz[4], ww[4], qq[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const bool ok = e + u < e1;
                        cc[u] = ok ? a.col[e + u] : row;
                        mm[u] = ok ? a.mA[e + u] : f4z;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const size_t ni = (size_t)cc[u] * Rp4 + c4;
                        zz[u] = Zr[ni];
                        ww[u] = Wr[ni];
                        qq[u] = Qr[ni];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        float4 qn;
                        acc_entry(mm[u], next_z(zz[u], ww[u], qq[u], al, be, qn));
                    }
                }
            }
            if (mine) {
                const size_t vi = (size_t)row * Rp4 + c4;
                const float4 zo = Zr[vi], wo = Wr[vi], qo = Qr[vi];
                const float4 po = P[vi], dd = Dv[vi];
                const float4 dgr = a.dg[row];
                float4 qn;
                const float4 zn = next_z(zo, wo, qo, al, be, qn);
                float pn[4], dn[4], wt[4];
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const float jr = gx[j] * sx[j].x + gy[j] * sy[j].x + gz[j] * sz[j].x;
                    const float ji = gx[j] * sx[j].y + gy[j] * sy[j].y + gz[j] * sz[j].y;
                    const float2 wv = make_float2(fmaf(-cn[j], ji, sA[j].x), fmaf(cn[j], jr, sA[j].y));   // w_k = A z_k
                    const float2 Dg = make_float2(dgr.x, cn[j] * (gx[j] * dgr.y + gy[j] * dgr.z + gz[j] * dgr.w));
                    const float2 wtj = cmulf(cinvf(Dg), wv);
                    const float2 zj = slot_of(zn, j), qj = slot_of(qn, j);
                    const float2 bp = cmulf(be[j], slot_of(po, j));
                    const float2 zoj = slot_of(zo, j);
                    const float2 pj = make_float2(zoj.x + bp.x, zoj.y + bp.y);            // p_{k-1}
                    const float2 ap = cmulf(al[j], pj);
                    const float2 dj = slot_of(dd, j);
                    pn[2 * j] = pj.x;
                    pn[2 * j + 1] = pj.y;
                    dn[2 * j] = dj.x + ap.x;
                    dn[2 * j + 1] = dj.y + ap.y;
                    wt[2 * j] = wtj.x;
                    wt[2 * j + 1] = wtj.y;
                    const float2 rj = cmulf(Dg, zj);        // r_k
                    const float2 qu = cmulf(Dg, qj);        // q_{k-1}
                    const float2 rz = cmulf(rj, zj), zw = cmulf(zj, wv), zq = cmulf(zj, qu), pq = cmulf(pj, qu);
                    kadd(v[j][0], rz.x);
                    kadd(v[j][1], rz.y);
                    kadd(v[j][2], rj.x * rj.x + rj.y * rj.y);
                    kadd(v[j][3], zw.x);
                    kadd(v[j][4], zw.y);
                    kadd(v[j][5], zq.x);
                    kadd(v[j][6], zq.y);
                    kadd(v[j][7], pq.x);
                    kadd(v[j][8], pq.y);
                }
                Zw[vi] = zn;
                Ww[vi] = make_float4(wt[0], wt[1], wt[2], wt[3]);
                Qw[vi] = qn;
                P[vi] = make_float4(pn[0], pn[1], pn[2], pn[3]);
                Dv[vi] = make_float4(dn[0], dn[1], dn[2], dn[3]);
            }
        }
        float2 o[2][kNV1];
        b.partials = (flip++ & 1u) ? part1 : part0;
        if (!reduce_rhs<LPR, kNV1>(v, o, b, chunk, r0, nb, bid, gen, smem)) return false;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (!act[j]) continue;
            const double2 rho = dd2(o[j][0], o[j][1]);
            const float nu = o[j][2].x + o[j][2].y;
            const double2 delta = dd2(o[j][3], o[j][4]);
            const double2 sigma = dd2(o[j][5], o[j][6]);
            const double2 mud = dd2(o[j][7], o[j][8]);
            const double rpn = rho_p[j].x * rho_p[j].x + rho_p[j].y * rho_p[j].y;
            const double2 beta = (it == 0 || !(rpn > 0.0)) ? make_double2(0.0, 0.0) : cdiv(rho, rho_p[j]);
            const double2 bs = cmul(beta, sigma), bbm = cmul(cmul(beta, beta), mud);
            const double2 mu = make_double2(delta.x + 2.0 * bs.x + bbm.x, delta.y + 2.0 * bs.y + bbm.y);
            const double mun = mu.x * mu.x + mu.y * mu.y, rhn = rho.x * rho.x + rho.y * rho.y;
            const bool ok = mun > 0.0 && isfinite(mun) && rhn > 0.0 && isfinite(rhn);
            const double2 alpha = ok ? cdiv(rho, mu) : make_double2(0.0, 0.0);
            al[j] = make_float2((float)alpha.x, (float)alpha.y);
            be[j] = ok ? make_float2((float)beta.x, (float)beta.y) : make_float2(0.f, 0.f);
            rho_p[j] = rho;
            rr2[j] = nu;
            rrmin[j] = fminf(rrmin[j], nu);
            if (nu < 0.25f * rrmark[j]) {
                rrmark[j] = nu;
                itmark[j] = it + 1;
            }
        }
        ++it;
    }
    return true;
}

// ------------------------------------------------------------------ kernel ----
// The stepper on one mesh, run by blocks bid = 0..nb-1 of a (sub-)grid whose
// blocks are all co-resident.
// kX: the optional paths (pseudo-periodic term, adjoint right-hand side w,
// per-step state saves) are compiled only into the kX = true kernels, so the
// plain stepper keeps the register allocation it has without them.
// kS: the inner FP32 solve runs the single-reduction COCG iteration (one grid-wide
// reduction per iteration, see below) instead of the two-reduction one.
template <int LPR, bool kX, bool kS>
__device__ __forceinline__ void batched_body(const MixArgs& a, const unsigned bid, const unsigned nb) {
    constexpr int G = 32 / LPR;  // rows per warp-unit
    constexpr int C = 2 * LPR;   // RHS per warp-unit
    constexpr int NVM = kS ? kNV1 : kNV;   // widest reduction of this variant
    __shared__ float2 smem[kWarpsB * 64 * NVM > kMaxRhs * NVM ? kWarpsB * 64 * NVM : kMaxRhs * NVM];
    const int lane = threadIdx.x & 31;
    const int gw = bid * kWarpsB + (threadIdx.x >> 5);
    const int total_warps = nb * kWarpsB;
    const int nchunks = a.Rp / C;
    const int chunk = gw % nchunks;
    const int slot = lane / LPR;
    const int r0 = chunk * C + (lane % LPR) * 2;  // this lane's first RHS
    const int c4 = r0 >> 1;                        // float4 index of the lane's 2 RHS inside a row
    const int Rp4 = a.Rp >> 1;                     // float4 per row
    const int ngroups = (a.n + G - 1) / G;
    // Row groups of this warp.  Interleaved: consecutive groups go to consecutive
    // warps of the whole grid.  Blocked: each block owns a contiguous range of
    // groups, so the neighbour rows its warps gather overlap and are reused in L1.
    int g0, gend, gstride;
    if (a.blocked) {
        g0 = (int)(((long long)ngroups * bid) / nb) + (threadIdx.x >> 5) / nchunks;
        gend = (int)(((long long)ngroups * (bid + 1)) / nb);
        gstride = kWarpsB / nchunks;
    } else {
        g0 = gw / nchunks;
        gend = ngroups;
        gstride = total_warps / nchunks;
    }
    unsigned gen = 0;
    if (a.stall) {   // bar[4] is never written: the wait runs out and the launch ends with DEV_TIMEOUT
        stalled_wait(a.bar + 4, a.status, a.wait_ns);
        return;
    }
    // per-lane RHS parameters
    double qd[2];
    float gx[2], gy[2], gz[2];
    int sq[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        qd[j] = a.qv[r0 + j];
        gx[j] = a.gv[(r0 + j) * 3 + 0];
        gy[j] = a.gv[(r0 + j) * 3 + 1];
        gz[j] = a.gv[(r0 + j) * 3 + 2];
        sq[j] = a.seqv[r0 + j];
    }
    // partial buffers alternate between consecutive reductions (see reduce_rhs)
    float2* const part0 = a.partials;
    float2* const part1 = a.partials + (size_t)nb * a.Rp * NVM;
    unsigned flip = 0;
    MixArgs b = a;
#define BT_REDUCE(V, OUT)                                                                  \
    do {                                                                                   \
        float2 o2_[2][kNV];                                                                \
        b.partials = (flip++ & 1u) ? part1 : part0;                                        \
        if (!reduce_rhs<LPR, kNV>(V, o2_, b, chunk, r0, nb, bid, gen, smem)) return;        \
        for (int j_ = 0; j_ < 2; ++j_)                                                     \
            for (int k_ = 0; k_ < kNV; ++k_) OUT[j_][k_] = o2_[j_][k_].x + o2_[j_][k_].y;  \
    } while (0)

    int dsel = 0;
    for (int step = 0; step < a.n_steps; ++step) {
        float cn[2], cs[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const double fnv = a.fnew[(size_t)sq[j] * a.sched_stride + step];
            const double fov = a.fold[(size_t)sq[j] * a.sched_stride + step];
            cn[j] = (float)(a.theta * qd[j] * fnv);
            cs[j] = (float)(a.theta * qd[j] * fnv + (1.0 - a.theta) * qd[j] * fov);  // cn + co
        }
        // ---- phase S, pass 1: r = -(S u + i (cn+co) Jg u) = b - A u_n in double-float
        //      for the lane's signal
        for (int g = g0; g < gend; g += gstride) {
            const int row = g * G + slot;
            if (row >= a.n) continue;
            DF sr[2], jx[2], jy[2], jz[2];  // [re/im]
#pragma unroll
            for (int c = 0; c < 2; ++c) sr[c] = jx[c] = jy[c] = jz[c] = DF{0.0f, 0.0f};
            const int e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
            for (int e = e0; e < e1; e += 4) {   // four gathers in flight, predicated tail
                int cc[4];
                float2 s2[4], uh[4], ul[4];
                float4 hi[4], lo[4];
                const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const bool ok = e + u < e1;
                    cc[u] = ok ? a.col[e + u] : row;
                    s2[u] = ok ? a.mS[e + u] : make_float2(0.f, 0.f);
                    hi[u] = ok ? a.mA[e + u] : z4;
                    lo[u] = ok ? a.mL[e + u] : z4;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    uh[u] = a.uh[(size_t)cc[u] * Rp4 + c4];
                    ul[u] = a.ul[(size_t)cc[u] * Rp4 + c4];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float uhv[2] = {uh[u].x, uh[u].y}, ulv[2] = {ul[u].x, ul[u].y};
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        df_fma(sr[c], s2[u].x, s2[u].y, uhv[c], ulv[c]);
                        df_fma(jx[c], hi[u].y, lo[u].y, uhv[c], ulv[c]);
                        df_fma(jy[c], hi[u].z, lo[u].z, uhv[c], ulv[c]);
                        df_fma(jz[c], hi[u].w, lo[u].w, uhv[c], ulv[c]);
                    }
                }
            }
            const size_t vi = (size_t)row * Rp4 + c4;
            DF jg[2];
#pragma unroll
            for (int c = 0; c < 2; ++c)
                jg[c] = df_add(df_add(df_scale(df_norm(jx[c]), gx[0]), df_scale(df_norm(jy[c]), gy[0])),
                               df_scale(df_norm(jz[c]), gz[0]));
            // -i cs (a + i b) = cs b - i cs a
            DF re = df_add(df_neg(df_norm(sr[0])), df_scale(jg[1], cs[0]));
            DF im = df_add(df_neg(df_norm(sr[1])), df_scale(jg[0], -cs[0]));
            if (kX && a.per_ptr && a.per_ptr[row] < a.per_ptr[row + 1]) {
                // pseudo-periodic mirror term of b, in FP64 (boundary rows only)
                const double2 bt = periodic_term(a, row, r0, c4, Rp4, qd[0] * a.Fint[(size_t)sq[0] * a.sched_stride + step]);
                const float bxh = (float)bt.x, byh = (float)bt.y;
                re = df_add(re, DF{bxh, (float)(bt.x - (double)bxh)});
                im = df_add(im, DF{byh, (float)(bt.y - (double)byh)});
            }
            if (kX && a.rhs_w && step == 0) {   // b = w from the zero state: r = w
                const double wv = a.w[row];
                const float wh = (float)wv;
                re = df_add(re, DF{wh, (float)(wv - (double)wh)});
            }
            a.rh[vi] = make_float2(re.h, im.h);
            a.rl[vi] = make_float2(re.l, im.l);
            if (a.extrap > 1 && step > 0) {
                // backward differences at u_n from the last step's correction d = hc:
                // t3 <- d - t1 - t2, t2 <- d - t1, t1 <- d (own row, own lane)
                const float2 dl = __ldcg(&a.hc[vi]), o1 = __ldcg(&a.t1[vi]);
                if (a.extrap > 2) {
                    const float2 o2 = __ldcg(&a.t2[vi]);
                    if (a.extrap > 3) a.t3[vi] = make_float2(dl.x - o1.x - o2.x, dl.y - o1.y - o2.y);
                    a.t2[vi] = make_float2(dl.x - o1.x, dl.y - o1.y);
                }
                a.t1[vi] = dl;
            }
        }
        // ---- phase S, pass 2 (same rows, same threads: no barrier): start from the
        //      extrapolated guess u_n + e, r -= A e in double-float; the FP32 inner solve
        //      starts from Re(r) (slot 0) and Im(r) (slot 1).  u itself is not written
        //      here (other threads may still gather u_n in pass 1): e is kept in hc
        //      and added to u by the first phase U.  e was formed by the last phase U
        //      of the previous step (ex); it is written inside this kernel, so it is
        //      read coherently (L2), never through the read-only path.
        const bool guess = a.extrap > 0 && step > 0;   // uniform over the grid
        KF red[2][kNV];
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < kNV; ++k) red[j][k] = KF{0.0f, 0.0f};
        for (int g = g0; g < gend; g += gstride) {
            const int row = g * G + slot;
            if (row >= a.n) continue;
            const size_t vi = (size_t)row * Rp4 + c4;
            DF ar[2], jx[2], jy[2], jz[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) ar[c] = jx[c] = jy[c] = jz[c] = DF{0.0f, 0.0f};
            float2 ev = make_float2(0.f, 0.f);
            if (guess) {
                const int e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
                for (int e = e0; e < e1; e += 4) {   // four gathers in flight, predicated tail
                    int cc[4];
                    float4 hi[4], lo[4];
                    float2 h1[4];
                    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const bool ok = e + u < e1;
                        cc[u] = ok ? a.col[e + u] : row;
                        hi[u] = ok ? a.mA[e + u] : z4;
                        lo[u] = ok ? a.mL[e + u] : z4;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) h1[u] = __ldcg(&a.ex[(size_t)cc[u] * Rp4 + c4]);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float2 en = h1[u];
                        const float ec[2] = {en.x, en.y};
#pragma unroll
                        for (int c = 0; c < 2; ++c) {
                            df_fma(ar[c], hi[u].x, lo[u].x, ec[c], 0.0f);
                            df_fma(jx[c], hi[u].y, lo[u].y, ec[c], 0.0f);
                            df_fma(jy[c], hi[u].z, lo[u].z, ec[c], 0.0f);
                            df_fma(jz[c], hi[u].w, lo[u].w, ec[c], 0.0f);
                        }
                    }
                }
                ev = __ldcg(&a.ex[vi]);
            }
            DF jg[2];
#pragma unroll
            for (int c = 0; c < 2; ++c)
                jg[c] = df_add(df_add(df_scale(df_norm(jx[c]), gx[0]), df_scale(df_norm(jy[c]), gy[0])),
                               df_scale(df_norm(jz[c]), gz[0]));
            // A e = A_re e + i cn Jg e
            const DF aer = df_add(df_norm(ar[0]), df_scale(jg[1], -cn[0]));
            const DF aei = df_add(df_norm(ar[1]), df_scale(jg[0], cn[0]));
            const float2 rh0 = a.rh[vi], rl0 = a.rl[vi];
            const DF re = df_add(DF{rh0.x, rl0.x}, df_neg(aer));
            const DF im = df_add(DF{rh0.y, rl0.y}, df_neg(aei));
            const float2 uhr = a.uh[vi];
            a.rh[vi] = make_float2(re.h, im.h);
            a.rl[vi] = make_float2(re.l, im.l);
            a.hc[vi] = ev;
            const float4 dgr = a.dg[row];
            const float wr = (float)a.w[row] * a.inv_k;
            const float2 dinv = cinvf(make_float2(dgr.x, cn[0] * (gx[0] * dgr.y + gy[0] * dgr.z + gz[0] * dgr.w)));
            const float2 z0 = make_float2(dinv.x * re.h, dinv.y * re.h);
            const float2 z1 = make_float2(dinv.x * im.h, dinv.y * im.h);
            a.ri[vi] = kS ? make_float4(0.f, 0.f, 0.f, 0.f) : make_float4(re.h, 0.f, im.h, 0.f);
            a.z[vi] = make_float4(z0.x, z0.y, z1.x, z1.y);
            a.p[vi] = make_float4(0.f, 0.f, 0.f, 0.f);
            a.q[vi] = make_float4(0.f, 0.f, 0.f, 0.f);
            a.dv[dsel][vi] = make_float4(0.f, 0.f, 0.f, 0.f);
            kadd(red[0][0], re.h * z0.x);
            kadd(red[0][1], re.h * z0.y);
            kadd(red[0][2], re.h * re.h);
            kadd(red[1][0], im.h * z1.x);
            kadd(red[1][1], im.h * z1.y);
            kadd(red[1][2], im.h * im.h);
            const float bn = (kX && a.rhs_w && step == 0) ? (float)(a.w[row] * a.w[row])
                                                    : wr * wr * (uhr.x * uhr.x + uhr.y * uhr.y);
            kadd(red[0][3], bn);
            kadd(red[1][3], bn);
        }
        float rs[2][kNV];
        BT_REDUCE(red, rs);
        float2 rho[2];
        float rr2[2], tolb2[2], rrs[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            rho[j] = make_float2(rs[j][0], rs[j][1]);
            rr2[j] = rs[j][2];
            rrs[j] = rs[j][2];
            tolb2[j] = a.rtol * a.rtol * rs[j][3];   // (rtol ||b||)^2
        }
        int sweep = 0, it_total = 0;
        bool failed = false;
        while (true) {
            // ---- inner FP32 Jacobi-COCG on A d = r (sweep start residual rrs)
            const float eps = (sweep == 0) ? a.eps_first : a.eps_next;
            float2 beta[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            // smallest residual of the sweep: a slot whose FP32 COCG residual grows
            // a.growth2 times above it (squared norms) is diverging (a near-breakdown of
            // the unconjugated form), and a slot whose residual has not halved (in
            // norm) for 64 iterations has reached FP32's attainable accuracy; either
            // ends its sweep, the double-float phase U measures the true residual and
            // the next sweep restarts from it
            float rrmin[2] = {rr2[0], rr2[1]};
            float rrmark[2] = {rr2[0], rr2[1]};
            int itmark[2] = {0, 0};
            bool act[2];
            int it = 0;
            if constexpr (kS) {
                if (!inner_single<LPR>(a, b, eps, rr2, rrs, tolb2, rrmin, rrmark, itmark, act, it, failed, step, sweep,
                                       cn, gx, gy, gz, dsel, g0, gend, gstride, slot, r0, c4, Rp4, chunk, nb, bid, gen,
                                       flip, part0, part1, smem))
                    return;
            } else {
            while (true) {
                // lane-local activity of its two RHS; the block-wide OR is the same in every
                // block (rr2 / rrs are grid-identical sums).  __syncthreads_or has barrier
                // semantics and no shared flag: a shared flag reset by one thread for the
                // next decision can race with a slow warp still reading the previous one.
#pragma unroll
                for (int j = 0; j < 2; ++j)
                    act[j] = (r0 + j < a.R) && rr2[j] > eps * eps * rrs[j] && rr2[j] > 0.09f * tolb2[j] &&
                             rr2[j] <= a.growth2 * rrmin[j] && it - itmark[j] < 64;
                if (!__syncthreads_or(act[0] || act[1])) break;
                if (it >= a.maxit) {
                    if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
#pragma unroll
                    for (int j = 0; j < 2; ++j)
                        if (bid == 0 && act[j]) {
                            a.diag[0] = 1.0f; a.diag[1] = (float)step; a.diag[2] = (float)sweep; a.diag[3] = (float)it;
                            a.diag[4] = rr2[j] / fmaxf(eps * eps * rrs[j], 1e-38f);
                            a.diag[5] = (float)(r0 / 2);
                        }
                    failed = true;
                    break;
                }
                // phase A: w = A z ; q = w + beta q ; p = z + beta p ; mu = p^T q
                KF mu[2][kNV];
#pragma unroll
                for (int j = 0; j < 2; ++j)
#pragma unroll
                    for (int k = 0; k < kNV; ++k) mu[j][k] = KF{0.0f, 0.0f};
                // a lane whose signal has converged in this sweep (or is padding) moves
                // no data: its step length is zero and phase U restarts its vectors
                const bool lane_active = act[0] || act[1];
                // With 8 or more lanes per row the lanes of a row share its column indices
                // and matrix values (one coalesced load, broadcast by shuffles), so all of a
                // row's neighbour gathers are in flight at once; every lane of the warp then
                // runs the same iterations (rows past the end are clamped, converged lanes
                // skip their own gathers and stores).
                constexpr bool kShared = (LPR >= 8);
                // (a warp whose lanes have all converged skips the rows: nothing it
                // would load is used)
                const bool warp_active = __any_sync(0xffffffffu, lane_active);
                for (int g = (kShared ? warp_active : lane_active) ? g0 : gend; g < gend; g += gstride) {
                    const int row_raw = g * G + slot;
                    if (!kShared && row_raw >= a.n) continue;
                    const bool row_ok = row_raw < a.n;
                    const int row = row_ok ? row_raw : a.n - 1;
                    const bool mine = row_ok && lane_active;   // this lane updates its slots
                    // the lane's two slots are the Re and Im parts of one signal: one
                    // gradient direction, so J_g = g.(Jx, Jy, Jz) is formed once per entry
                    float2 sA[2], sJ[2];
#pragma unroll
                    for (int j = 0; j < 2; ++j) sA[j] = sJ[j] = make_float2(0.f, 0.f);
                    const int e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
                    auto acc_entry = [&](const float4 m, const float4 zz) {
                        const float2 zj[2] = {make_float2(zz.x, zz.y), make_float2(zz.z, zz.w)};
                        const float jg = fmaf(m.w, gz[0], fmaf(m.z, gy[0], m.y * gx[0]));
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            sA[j].x = fmaf(m.x, zj[j].x, sA[j].x); sA[j].y = fmaf(m.x, zj[j].y, sA[j].y);
                            sJ[j].x = fmaf(jg, zj[j].x, sJ[j].x); sJ[j].y = fmaf(jg, zj[j].y, sJ[j].y);
                        }
                    };
                    const size_t vi = (size_t)row * Rp4 + c4;
                    const float4 f4z = make_float4(0.f, 0.f, 0.f, 0.f);
                    const float4 po = mine ? a.p[vi] : f4z, qo = mine ? a.q[vi] : f4z;
                    if constexpr (kShared) {
                        // windows of 16 entries: lane gl of the row's group loads entries gl,
                        // gl + LPR, ... of the window, then 16 gathers go out together
                        constexpr int W = 16;
                        constexpr int K = (W + LPR - 1) / LPR;
                        const int gl = lane % LPR;
                        const int nn = e1 - e0;
                        const int nmax = __reduce_max_sync(0xffffffffu, nn);
                        for (int off = 0; off < nmax; off += W) {
                            int my_c[K];
                            float4 my_m[K];
#pragma unroll
                            for (int k = 0; k < K; ++k) {
                                const int u = gl + k * LPR;
                                const bool ok = u < W && off + u < nn;
                                my_c[k] = ok ? a.col[e0 + off + u] : row;
                                my_m[k] = ok ? a.mA[e0 + off + u] : f4z;
                            }
                            float4 zz[W];
#pragma unroll
                            for (int u = 0; u < W; ++u) {
                                const int c = __shfl_sync(0xffffffffu, my_c[u / LPR], u % LPR, LPR);
                                zz[u] = mine ? a.z[(size_t)c * Rp4 + c4] : f4z;
                            }
#pragma unroll
                            for (int u = 0; u < W; ++u) {
                                float4 m;
                                m.x = __shfl_sync(0xffffffffu, my_m[u / LPR].x, u % LPR, LPR);
                                m.y = __shfl_sync(0xffffffffu, my_m[u / LPR].y, u % LPR, LPR);
                                m.z = __shfl_sync(0xffffffffu, my_m[u / LPR].z, u % LPR, LPR);
                                m.w = __shfl_sync(0xffffffffu, my_m[u / LPR].w, u % LPR, LPR);
                                acc_entry(m, zz[u]);
                            }
                        }
                    } else {
                        // eight independent neighbour gathers in flight per lane; the tail of
                        // a row is predicated (a missing entry reads the own row times zero)
                        for (int e = e0; e < e1; e += 8) {
                            int cc[8];
                            float4 mm[8], zz[8];
#pragma unroll
                            for (int u = 0; u < 8; ++u) {
                                const bool ok = e + u < e1;
                                cc[u] = ok ? a.col[e + u] : row;
                                mm[u] = ok ? a.mA[e + u] : f4z;
                            }
#pragma unroll
                            for (int u = 0; u < 8; ++u) zz[u] = a.z[(size_t)cc[u] * Rp4 + c4];
#pragma unroll
                            for (int u = 0; u < 8; ++u) acc_entry(mm[u], zz[u]);
                        }
                    }
                    const float4 zo = mine ? a.z[vi] : f4z;
                    const float zov[4] = {zo.x, zo.y, zo.z, zo.w}, pov[4] = {po.x, po.y, po.z, po.w},
                                qov[4] = {qo.x, qo.y, qo.z, qo.w};
                    float pn[4], qn[4];
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const float2 wv = make_float2(fmaf(-cn[j], sJ[j].y, sA[j].x), fmaf(cn[j], sJ[j].x, sA[j].y));
                        const float2 bp = cmulf(beta[j], make_float2(pov[2 * j], pov[2 * j + 1]));
                        const float2 bq = cmulf(beta[j], make_float2(qov[2 * j], qov[2 * j + 1]));
                        pn[2 * j] = zov[2 * j] + bp.x;
                        pn[2 * j + 1] = zov[2 * j + 1] + bp.y;
                        qn[2 * j] = wv.x + bq.x;
                        qn[2 * j + 1] = wv.y + bq.y;
                        const float2 pq = cmulf(make_float2(pn[2 * j], pn[2 * j + 1]), make_float2(qn[2 * j], qn[2 * j + 1]));
                        if (mine) {
                            kadd(mu[j][0], pq.x);
                            kadd(mu[j][1], pq.y);
                        }
                    }
                    if (mine) {
                        a.p[vi] = make_float4(pn[0], pn[1], pn[2], pn[3]);
                        a.q[vi] = make_float4(qn[0], qn[1], qn[2], qn[3]);
                    }
                }
                float ms[2][kNV];
                BT_REDUCE(mu, ms);
                float2 alpha[2];
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const float2 m2 = make_float2(ms[j][0], ms[j][1]);
                    // inactive or broken-down slots take no step (the residual stays put;
                    // the outer check reports it if it never converges)
                    alpha[j] = (act[j] && cnonzero(m2) && cnonzero(rho[j])) ? cdivf(rho[j], m2)
                                                                           : make_float2(0.f, 0.f);
                }
                // phase B: d += alpha p ; r -= alpha q ; z = D^-1 r
                KF rb[2][kNV];
#pragma unroll
                for (int j = 0; j < 2; ++j)
#pragma unroll
                    for (int k = 0; k < kNV; ++k) rb[j][k] = KF{0.0f, 0.0f};
                auto phase_b_row = [&](size_t vi, const float4 pv, const float4 qv, const float4 dv, const float4 rv,
                                       const float4 dgr) {
                    const float pvv[4] = {pv.x, pv.y, pv.z, pv.w}, qvv[4] = {qv.x, qv.y, qv.z, qv.w};
                    float dn[4] = {dv.x, dv.y, dv.z, dv.w}, rn[4] = {rv.x, rv.y, rv.z, rv.w}, zn[4];
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const float2 ap = cmulf(alpha[j], make_float2(pvv[2 * j], pvv[2 * j + 1]));
                        const float2 aq = cmulf(alpha[j], make_float2(qvv[2 * j], qvv[2 * j + 1]));
                        dn[2 * j] += ap.x;
                        dn[2 * j + 1] += ap.y;
                        rn[2 * j] -= aq.x;
                        rn[2 * j + 1] -= aq.y;
                        const float2 dinv =
                            cinvf(make_float2(dgr.x, cn[j] * (gx[j] * dgr.y + gy[j] * dgr.z + gz[j] * dgr.w)));
                        const float2 zz = cmulf(dinv, make_float2(rn[2 * j], rn[2 * j + 1]));
                        zn[2 * j] = zz.x;
                        zn[2 * j + 1] = zz.y;
                        const float2 rz = cmulf(make_float2(rn[2 * j], rn[2 * j + 1]), zz);
                        kadd(rb[j][0], rz.x);
                        kadd(rb[j][1], rz.y);
                        kadd(rb[j][2], rn[2 * j] * rn[2 * j] + rn[2 * j + 1] * rn[2 * j + 1]);
                    }
                    a.dv[dsel][vi] = make_float4(dn[0], dn[1], dn[2], dn[3]);
                    a.ri[vi] = make_float4(rn[0], rn[1], rn[2], rn[3]);
                    a.z[vi] = make_float4(zn[0], zn[1], zn[2], zn[3]);
                };
                // two rows per pass: both rows' loads are in flight together (same
                // accumulation order as one row at a time)
                for (int g = lane_active ? g0 : gend; g < gend; g += 2 * gstride) {
                    const int rowA = g * G + slot, g2 = g + gstride, rowB = g2 * G + slot;
                    const bool okA = rowA < a.n, okB = g2 < gend && rowB < a.n;
                    const size_t viA = (size_t)(okA ? rowA : 0) * Rp4 + c4, viB = (size_t)(okB ? rowB : 0) * Rp4 + c4;
                    const float4 f4z = make_float4(0.f, 0.f, 0.f, 0.f);
                    const float4 pA = okA ? a.p[viA] : f4z, qA = okA ? a.q[viA] : f4z;
                    const float4 dA = okA ? a.dv[dsel][viA] : f4z, rA = okA ? a.ri[viA] : f4z;
                    const float4 gA = okA ? a.dg[rowA] : f4z;
                    const float4 pB = okB ? a.p[viB] : f4z, qB = okB ? a.q[viB] : f4z;
                    const float4 dB = okB ? a.dv[dsel][viB] : f4z, rB = okB ? a.ri[viB] : f4z;
                    const float4 gB = okB ? a.dg[rowB] : f4z;
                    if (okA) phase_b_row(viA, pA, qA, dA, rA, gA);
                    if (okB) phase_b_row(viB, pB, qB, dB, rB, gB);
                }
                float rbs[2][kNV];
                BT_REDUCE(rb, rbs);
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const float2 rn2 = make_float2(rbs[j][0], rbs[j][1]);
                    beta[j] = (act[j] && cnonzero(rho[j])) ? cdivf(rn2, rho[j]) : make_float2(0.f, 0.f);
                    if (act[j]) {
                        rho[j] = rn2;
                        rr2[j] = rbs[j][2];
                        rrmin[j] = fminf(rrmin[j], rr2[j]);
                        if (rr2[j] < 0.25f * rrmark[j]) {
                            rrmark[j] = rr2[j];
                            itmark[j] = it + 1;
                        }
                    }
                }
                ++it;
            }
            }   // kS
            it_total += it;
            if (failed) break;
            // ---- phase U: d = d_re-part + i d_im-part ; u += d ; r -= A d (double-float);
            //      restart the inner slots from Re(r), Im(r)
            KF ru[2][kNV];
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int k = 0; k < kNV; ++k) ru[j][k] = KF{0.0f, 0.0f};
            for (int g = g0; g < gend; g += gstride) {
                const int row = g * G + slot;
                if (row >= a.n) continue;
                DF ar[2], jx[2], jy[2], jz[2];
#pragma unroll
                for (int c = 0; c < 2; ++c) ar[c] = jx[c] = jy[c] = jz[c] = DF{0.0f, 0.0f};
                const int e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
                for (int e = e0; e < e1; e += 4) {   // four gathers in flight, predicated tail
                    int cc[4];
                    float4 hi[4], lo[4], dd[4];
                    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const bool ok = e + u < e1;
                        cc[u] = ok ? a.col[e + u] : row;
                        hi[u] = ok ? a.mA[e + u] : z4;
                        lo[u] = ok ? a.mL[e + u] : z4;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) dd[u] = a.dv[dsel][(size_t)cc[u] * Rp4 + c4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float dc[2] = {dd[u].x - dd[u].w, dd[u].y + dd[u].z};  // d0 + i d1
#pragma unroll
                        for (int c = 0; c < 2; ++c) {
                            df_fma(ar[c], hi[u].x, lo[u].x, dc[c], 0.0f);
                            df_fma(jx[c], hi[u].y, lo[u].y, dc[c], 0.0f);
                            df_fma(jy[c], hi[u].z, lo[u].z, dc[c], 0.0f);
                            df_fma(jz[c], hi[u].w, lo[u].w, dc[c], 0.0f);
                        }
                    }
                }
                const size_t vi = (size_t)row * Rp4 + c4;
                const float4 dgr = a.dg[row];
                const float2 rh = a.rh[vi], rl = a.rl[vi], uh = a.uh[vi], ul = a.ul[vi];
                const float4 dd = a.dv[dsel][vi];
                const float dco[2] = {dd.x - dd.w, dd.y + dd.z};
                DF jg[2];
#pragma unroll
                for (int c = 0; c < 2; ++c)
                    jg[c] = df_add(df_add(df_scale(df_norm(jx[c]), gx[0]), df_scale(df_norm(jy[c]), gy[0])),
                                   df_scale(df_norm(jz[c]), gz[0]));
                // A d = A_re d + i cn Jg d
                const DF adr = df_add(df_norm(ar[0]), df_scale(jg[1], -cn[0]));
                const DF adi = df_add(df_norm(ar[1]), df_scale(jg[0], cn[0]));
                const DF nr = df_add(DF{rh.x, rl.x}, df_neg(adr));
                const DF ni = df_add(DF{rh.y, rl.y}, df_neg(adi));
                // hc holds this step's total correction; in the first sweep it is the
                // guess offset e, which enters u here
                const float2 hc = a.hc[vi];
                const float2 eo = (sweep == 0) ? hc : make_float2(0.f, 0.f);
                const DF u_re = df_add(df_add(DF{uh.x, ul.x}, DF{eo.x, 0.0f}), DF{dco[0], 0.0f});
                const DF u_im = df_add(df_add(DF{uh.y, ul.y}, DF{eo.y, 0.0f}), DF{dco[1], 0.0f});
                a.rh[vi] = make_float2(nr.h, ni.h);
                a.rl[vi] = make_float2(nr.l, ni.l);
                a.uh[vi] = make_float2(u_re.h, u_im.h);
                a.ul[vi] = make_float2(u_re.l, u_im.l);
                const float2 dlt = make_float2(hc.x + dco[0], hc.y + dco[1]);
                a.hc[vi] = dlt;
                if (a.extrap > 0) {
                    // the next step's offset: Newton backward extrapolation of order hp,
                    // e = hp d - (hp-1) t1 - (hp-2) t2 - (hp-3) t3 with d = u_{n+1} - u_n and
                    // t1..t3 the differences at u_n (x0 = 3u_{n+1} - 3u_n + u_{n-1} for hp = 2)
                    const int hp = min(step + 1, a.extrap);
                    float2 E = make_float2((float)hp * dlt.x, (float)hp * dlt.y);
                    if (hp >= 2) {
                        const float2 o1 = __ldcg(&a.t1[vi]);
                        E.x = fmaf(-(float)(hp - 1), o1.x, E.x);
                        E.y = fmaf(-(float)(hp - 1), o1.y, E.y);
                    }
                    if (hp >= 3) {
                        const float2 o2 = __ldcg(&a.t2[vi]);
                        E.x = fmaf(-(float)(hp - 2), o2.x, E.x);
                        E.y = fmaf(-(float)(hp - 2), o2.y, E.y);
                    }
                    if (hp >= 4) {
                        const float2 o3 = __ldcg(&a.t3[vi]);
                        E.x -= o3.x;
                        E.y -= o3.y;
                    }
                    a.ex[vi] = E;
                }
                const float2 dinv = cinvf(make_float2(dgr.x, cn[0] * (gx[0] * dgr.y + gy[0] * dgr.z + gz[0] * dgr.w)));
                const float2 z0 = make_float2(dinv.x * nr.h, dinv.y * nr.h);
                const float2 z1 = make_float2(dinv.x * ni.h, dinv.y * ni.h);
                a.ri[vi] = kS ? make_float4(0.f, 0.f, 0.f, 0.f) : make_float4(nr.h, 0.f, ni.h, 0.f);
                a.z[vi] = make_float4(z0.x, z0.y, z1.x, z1.y);
                a.p[vi] = make_float4(0.f, 0.f, 0.f, 0.f);
                a.q[vi] = make_float4(0.f, 0.f, 0.f, 0.f);
                a.dv[dsel ^ 1][vi] = make_float4(0.f, 0.f, 0.f, 0.f);
                kadd(ru[0][0], nr.h * z0.x);
                kadd(ru[0][1], nr.h * z0.y);
                kadd(ru[0][2], nr.h * nr.h);
                kadd(ru[1][0], ni.h * z1.x);
                kadd(ru[1][1], ni.h * z1.y);
                kadd(ru[1][2], ni.h * ni.h);
            }
            float rus[2][kNV];
            BT_REDUCE(ru, rus);
            dsel ^= 1;
            ++sweep;
            bool more = false;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                rho[j] = make_float2(rus[j][0], rus[j][1]);
                rr2[j] = rus[j][2];
                rrs[j] = rus[j][2];
            }
            // the lane's two slots are Re and Im of one signal: ||r||^2 = sum of both
            if (r0 < a.R && rr2[0] + rr2[1] > tolb2[0]) more = true;
            if (!__syncthreads_or(more)) break;
            if (sweep >= a.max_sweeps) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
                if (bid == 0 && r0 < a.R && rr2[0] + rr2[1] > tolb2[0]) {
                    a.diag[0] = 2.0f; a.diag[1] = (float)step; a.diag[2] = (float)sweep; a.diag[3] = (float)it_total;
                    a.diag[4] = (rr2[0] + rr2[1]) / fmaxf(tolb2[0], 1e-38f); a.diag[5] = (float)(r0 / 2);
                }
                failed = true;
                break;
            }
        }
        if (bid == 0 && threadIdx.x == 0) {
            a.iters[step] = it_total;
            a.sweeps[step] = sweep;
        }
        if (failed) return;
        if (kX && a.save_h && (step + 1) % a.save_every == 0) {
            // every lane copies its own (row, signal) entries, which it wrote itself in phase U
            const size_t off = (size_t)((step + 1) / a.save_every - 1) * a.n * Rp4;
            for (int g = g0; g < gend; g += gstride) {
                const int row = g * G + slot;
                if (row >= a.n) continue;
                const size_t vi = (size_t)row * Rp4 + c4;
                a.save_h[off + vi] = a.uh[vi];
                a.save_l[off + vi] = a.ul[vi];
            }
        }
    }
#undef BT_REDUCE
    // ---- signal: FP64 sums of w Re(u) per RHS and compartment (lanes own their RHS)
    double acc[2][1 + kMaxCompartments];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int k = 0; k <= kMaxCompartments; ++k) acc[j][k] = 0.0;
    for (int g = g0; g < gend; g += gstride) {
        const int row = g * G + slot;
        if (row >= a.n) continue;
        const size_t vi = (size_t)row * Rp4 + c4;
        const float2 uh = a.uh[vi], ul = a.ul[vi];
        const double wr = a.w[row];
        const int cm = a.rcomp[row];
        const double v0 = wr * ((double)uh.x + (double)ul.x);
        acc[0][0] += v0;
#pragma unroll
        for (int k = 0; k < kMaxCompartments; ++k)
            if (k == cm) acc[0][1 + k] += v0;
    }
    // deterministic: combine the row slots by shuffles, stage per-warp partials,
    // then sum the warps of each RHS chunk in warp order
#pragma unroll
    for (int o = 16; o >= LPR; o >>= 1)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k <= kMaxCompartments; ++k) acc[j][k] += __shfl_xor_sync(0xffffffffu, acc[j][k], o);
    double* wp = a.sigpart;  // [total_warps][C][1+kMaxCompartments], not shared with the reductions
    if (lane < LPR) {
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k <= kMaxCompartments; ++k)
                wp[((size_t)gw * C + lane * 2 + j) * (1 + kMaxCompartments) + k] = acc[j][k];
    }
    if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return;
    // grid thread t finishes (RHS r, value k): sum over warps of r's chunk in warp order
    const int gt = bid * blockDim.x + threadIdx.x;
    for (int t = gt; t < a.Rp * (1 + kMaxCompartments); t += nb * blockDim.x) {
        const int r = t / (1 + kMaxCompartments), k = t % (1 + kMaxCompartments);
        const int c = r / C, o = r % C;
        double s = 0.0;
        for (int wv = c; wv < total_warps; wv += nchunks)
            s += __ldcg(&wp[((size_t)wv * C + o) * (1 + kMaxCompartments) + k]);
        a.sig[t] = s;
    }
}

template <int LPR, bool kX, bool kS>
__global__ void __maxnreg__(kS ? 128 : 120) k_batched(MixArgs a) {
    batched_body<LPR, kX, kS>(a, blockIdx.x, gridDim.x);
}

// Several meshes in one cooperative launch: blocks first[m] .. first[m+1]-1 form
// the sub-grid of mesh m, which runs its own stepper with its own barrier
// counters and reductions; meshes never wait for one another.
template <int LPR, bool kX, bool kS>
__global__ void __maxnreg__(kS ? 128 : 120) k_batched_multi(const MixArgs* __restrict__ args, const int* __restrict__ first,
                                                 int n_meshes) {
    __shared__ MixArgs s_a;
    __shared__ int s_m;
    if (threadIdx.x == 0) {
        int m = 0;
        while (m + 1 < n_meshes && (int)blockIdx.x >= first[m + 1]) ++m;
        s_m = m;
        s_a = args[m];
    }
    __syncthreads();
    const int m = s_m;
    batched_body<LPR, kX, kS>(s_a, blockIdx.x - first[m], first[m + 1] - first[m]);
}

// Pack the double-float matrix copies and the row data once per assembly/theta/dt.
__global__ void k_pack_mixed(int64_t nnz, const double* __restrict__ M, const double* __restrict__ K,
                             const double* __restrict__ T, const double* __restrict__ R,
                             const double* __restrict__ Jx, const double* __restrict__ Jy,
                             const double* __restrict__ Jz, double inv_k, double theta,
                             const double* __restrict__ PB, float4* __restrict__ mA, float4* __restrict__ mL,
                             float2* __restrict__ mS) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    // S = A_re - B_re: the implicit matrix holds theta * PB, the explicit one does not
    const double S = K[e] + T[e] + R[e] + (PB ? theta * PB[e] : 0.0);
    const double A = M[e] * inv_k + theta * (K[e] + T[e] + R[e]) + (PB ? theta * PB[e] : 0.0);
    const double v[4] = {A, Jx[e], Jy[e], Jz[e]};
    float h[4], l[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        h[k] = (float)v[k];
        l[k] = (float)(v[k] - (double)h[k]);
    }
    mA[e] = make_float4(h[0], h[1], h[2], h[3]);
    mL[e] = make_float4(l[0], l[1], l[2], l[3]);
    const float sh = (float)S;
    mS[e] = make_float2(sh, (float)(S - (double)sh));
}

__global__ void k_rows_mixed(int64_t n, int32_t Rp, int32_t R, const int32_t* __restrict__ diag_pos,
                             const float4* __restrict__ mA, const double* __restrict__ wsrc,
                             const int32_t* __restrict__ comp, const int32_t* __restrict__ dof_vertex,
                             const double* __restrict__ u0, float4* __restrict__ dg, double* __restrict__ w,
                             int32_t* __restrict__ rcomp, float2* __restrict__ uh, float2* __restrict__ ul) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dg[i] = mA[diag_pos[i]];
    w[i] = wsrc[i];
    rcomp[i] = comp[i];
    const double v = u0 ? u0[dof_vertex[i]] : 1.0;
    const float h = (float)v;
    const float l = (float)(v - (double)h);
    const int ns = Rp / 2;  // signals per row: slots 2s, 2s+1 are Re / Im parts of signal s
    for (int sg = 0; sg < ns; ++sg) {
        const bool live = 2 * sg < R;
        uh[(size_t)i * ns + sg] = make_float2(live ? h : 0.f, 0.f);
        ul[(size_t)i * ns + sg] = make_float2(live ? l : 0.f, 0.f);
    }
}

namespace {

using KFn = void (*)(MixArgs);
using KFnMulti = void (*)(const MixArgs*, const int*, int);

template <bool kX, bool kS>
KFnMulti kernel_multi_lpr(int lpr) {
    switch (lpr) {
        case 1: return k_batched_multi<1, kX, kS>;
        case 2: return k_batched_multi<2, kX, kS>;
        case 4: return k_batched_multi<4, kX, kS>;
        case 8: return k_batched_multi<8, kX, kS>;
        case 16: return k_batched_multi<16, kX, kS>;
        default: return k_batched_multi<32, kX, kS>;
    }
}

template <bool kX, bool kS>
KFn kernel_lpr(int lpr) {
    switch (lpr) {
        case 1: return k_batched<1, kX, kS>;
        case 2: return k_batched<2, kX, kS>;
        case 4: return k_batched<4, kX, kS>;
        case 8: return k_batched<8, kX, kS>;
        case 16: return k_batched<16, kX, kS>;
        default: return k_batched<32, kX, kS>;
    }
}

// The optional paths (extras) run the two-reduction inner iteration; the plain
// stepper runs the single-reduction one when `single`.
KFn kernel_for(int lpr, bool extras, bool single) {
    return extras ? kernel_lpr<true, false>(lpr) : (single ? kernel_lpr<false, true>(lpr) : kernel_lpr<false, false>(lpr));
}

KFnMulti kernel_multi_for(int lpr, bool extras, bool single) {
    return extras ? kernel_multi_lpr<true, false>(lpr)
                  : (single ? kernel_multi_lpr<false, true>(lpr) : kernel_multi_lpr<false, false>(lpr));
}

int ceil_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

// Padded RHS count for chunk C = 2*LPR: the number of chunks is rounded up to
// a power of two <= 8, so every block of 8 warps covers every chunk equally.
int padded_rhs(int R, int lpr) {
    const int C = 2 * lpr;
    const int nch = ceil_pow2((R + C - 1) / C);
    return (nch <= kWarpsB) ? C * nch : -1;
}

// Valid lanes-per-row for a batch of R: C = 2*LPR no larger than the padded
// batch needs, and at most 8 chunks.
std::vector<int> lpr_candidates(int R) {
    std::vector<int> out;
    const int Rp2 = std::max(2, ceil_pow2(R));
    for (int lpr = 1; lpr <= 32; lpr <<= 1) {
        if (2 * lpr > Rp2) break;
        if (padded_rhs(R, lpr) > 0) out.push_back(lpr);
    }
    return out;
}

}  // namespace

static void map_status_mixed(int st) {
    switch (st) {
        case DEV_OK: return;
        case DEV_TIMEOUT: throw Error(BT_ERR_TIMEOUT, "mixed stepper: a grid barrier wait ran out of time");
        case DEV_NOT_CONVERGED:
            throw Error(BT_ERR_NOT_CONVERGED, "mixed stepper: inner COCG or refinement did not converge");
        default: throw Error(BT_ERR_CUDA, "mixed stepper: device status " + std::to_string(st));
    }
}

// Launch one batch (R <= 512 signals) with the given geometry; n_steps may be
// truncated for tuning.  Returns the device time of the stepper kernel (ms).
// Warp-units of a batch on this mesh: row groups x RHS chunks.  A (sub-)grid of
// more than units/8 blocks would leave blocks idle.
static int blocks_needed(const bt_ctx* ctx, int R, int lpr) {
    const int Rp = padded_rhs(R, lpr);
    const int G = 32 / lpr;
    const int64_t units = ((ctx->mesh.n_dofs + G - 1) / G) * (Rp / (2 * lpr));
    return (int)std::max<int64_t>(1, (units + kWarpsB - 1) / kWarpsB);
}

// Buffers, initial state and kernel arguments of one batch of R slots on one
// mesh, for a (sub-)grid of nb blocks; nothing is launched.  n_steps may be
// truncated for tuning.
static MixArgs prepare_batch(bt_ctx* ctx, SolverMixed& W, int R, int lpr, int nb, int blocked, int n_steps,
                             double rtol, int maxit, const double* d_u0, bool single) {
    Mesh& m = ctx->mesh;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    BT_REQUIRE(R >= 1 && R <= kMaxRhs && (lpr == 1 || lpr == 2 || lpr == 4 || lpr == 8 || lpr == 16 || lpr == 32),
               BT_ERR_INVALID, "mixed stepper: invalid batch geometry");
    const int Rp = padded_rhs(R, lpr);
    BT_REQUIRE(Rp >= R && Rp <= kMaxRhs && (Rp / (2 * lpr)) <= kWarpsB && (kWarpsB % (Rp / (2 * lpr))) == 0,
               BT_ERR_INVALID, "mixed stepper: invalid RHS padding");
    BT_REQUIRE(nb >= 1, BT_ERR_INVALID, "mixed stepper: empty grid");
    // partials: two alternating float buffers [nb][Rp][NV] for the widest reduction NV
    const int nvm = single ? kNV1 : kNV;
    W.partials.alloc((size_t)2 * nb * Rp * nvm);
    W.sigpart.alloc((size_t)nb * kWarpsB * 64 * (1 + kMaxCompartments));
    W.fin.alloc((size_t)Rp * nvm);
    const size_t nv = (size_t)m.n_dofs * Rp;
    for (auto* v : {&W.d0, &W.d1, &W.ri, &W.z, &W.p, &W.q}) v->alloc(nv);        // per slot
    if (single)
        for (auto* v : {&W.z1, &W.w1, &W.q1}) v->alloc(nv);                     // second buffers of z, w~, q~
    for (auto* v : {&W.uh, &W.ul, &W.rh, &W.rl, &W.hc, &W.t1, &W.t2, &W.t3, &W.ex}) v->alloc(nv / 2);   // per signal
    for (auto* v : {&W.hc, &W.t1, &W.t2, &W.t3, &W.ex}) v->zero(s);
    W.sig.alloc((size_t)Rp * (1 + kMaxCompartments));
    W.bar.alloc(6);   // [0], [1]: barrier / last-block arrival and release; [2..3]: 64-bit arrival counter;
                      // [4]: never written (stalled_wait)
    W.status.alloc(1);
    W.diag.alloc(8);
    W.diag.zero(s);
    k_rows_mixed<<<(unsigned)((m.n_dofs + 255) / 256), 256, 0, s>>>(m.n_dofs, Rp, R, m.diag_pos, W.mA, ctx->mat.w,
                                                                    m.dof_comp, m.dof_vertex, d_u0, W.dg, W.w,
                                                                    W.rcomp, W.uh, W.ul);
    BT_CUDA(cudaGetLastError());
    W.bar.zero(s);
    W.status.zero(s);
    MixArgs a;
    a.n = (int32_t)m.n_dofs;
    a.Rp = Rp;
    a.R = R;
    a.row_ptr = m.row_ptr;
    a.col = m.col;
    a.mA = W.mA;
    a.mL = W.mL;
    a.mS = W.mS;
    {
        const Periodic& P = ctx->per;
        a.per_ptr = P.on ? P.ptr.p : nullptr;
        a.per_col = P.col.p;
        a.per_val = P.val.p;
        a.Fint = P.on ? W.Fint.p : nullptr;
        a.gvd = W.gvd.p;
        a.theta_d = S.theta;
        a.growth2 = (float)ctx->opt_mixed_growth2;
        a.rhs_w = 0;
        a.save_every = 1;
        a.save_h = nullptr;
        a.save_l = nullptr;
        BT_REQUIRE(!P.on || (W.Fint.p && W.gvd.p), BT_ERR_STATE, "periodic phase schedule missing");
    }
    a.dg = W.dg;
    a.w = W.w;
    a.rcomp = W.rcomp;
    a.uh = W.uh.p;
    a.ul = W.ul.p;
    a.rh = W.rh.p;
    a.rl = W.rl.p;
    a.dv[0] = reinterpret_cast<float4*>(W.d0.p);
    a.dv[1] = reinterpret_cast<float4*>(W.d1.p);
    a.ri = reinterpret_cast<float4*>(W.ri.p);
    a.z = reinterpret_cast<float4*>(W.z.p);
    a.p = reinterpret_cast<float4*>(W.p.p);
    a.q = reinterpret_cast<float4*>(W.q.p);
    a.z1 = single ? reinterpret_cast<float4*>(W.z1.p) : nullptr;
    a.w1 = single ? reinterpret_cast<float4*>(W.w1.p) : nullptr;
    a.q1 = single ? reinterpret_cast<float4*>(W.q1.p) : nullptr;
    a.hc = W.hc.p;
    a.t1 = W.t1.p;
    a.t2 = W.t2.p;
    a.t3 = W.t3.p;
    a.ex = W.ex.p;
    a.extrap = ctx->opt_mixed_extrapolate;
    a.partials = W.partials;
    a.fin = W.fin;
    a.sigpart = W.sigpart;
    a.bar = W.bar;
    a.status = W.status;
    a.fnew = W.fnew;
    a.fold = W.fold;
    a.qv = W.qv;
    a.gv = W.gv;
    a.seqv = W.seqv;
    a.n_steps = n_steps;
    a.sched_stride = S.n_steps;
    BT_REQUIRE(n_steps >= 1 && n_steps <= S.n_steps, BT_ERR_INVALID, "mixed stepper: bad step count");
    a.maxit = maxit;
    a.max_sweeps = ctx->opt_mixed_max_sweeps;
    a.theta = (float)S.theta;
    a.inv_k = (float)(1.0 / S.dt);
    a.rtol = (float)rtol;
    a.eps_first = (float)ctx->opt_mixed_eps_first;
    a.eps_next = (float)ctx->opt_mixed_eps_next;
    {
        // Grid sums: two stages when one block would read too many partials; every
        // block summing them itself when that is at most 20 loads a thread (it saves
        // the publish / release / read-back round trips of the last-block form: 20 %
        // on the 20^3 box, 1-2 % on the 40^3 box; slower from ~10k partial values)
        const size_t nvals = (size_t)nb * Rp * nvm;
        a.reduce_mode = nvals > 12288 ? 2 : (ctx->opt_mixed_reduce >= 0 ? ctx->opt_mixed_reduce
                                                                         : (nvals <= 5120 ? 1 : 0));
    }
    a.blocked = blocked;
    a.iters = W.iters;
    a.sweeps = W.sweeps;
    a.wait_ns = ctx->opt_wait_ns;
    a.stall = ctx->opt_stall_first_wait;
    a.sig = W.sig;
    a.diag = W.diag;
    {
        const void* need_ptrs[] = {a.row_ptr, a.col, a.mA, a.mL, a.mS, a.dg, a.w, a.rcomp, a.uh, a.ul, a.rh, a.rl,
                                   a.dv[0], a.dv[1], a.ri, a.z, a.p, a.q, a.hc, a.t1, a.t2, a.t3, a.ex, a.partials, a.fin, a.sigpart, a.bar,
                                   a.status, a.fnew, a.fold, a.qv, a.gv, a.seqv, a.iters, a.sweeps, a.sig, a.diag};
        for (const void* ptr : need_ptrs)
            BT_REQUIRE(ptr != nullptr, BT_ERR_STATE, "mixed stepper: a device buffer is not allocated");
    }
    W.Rp = Rp;
    W.nb = nb;
    return a;
}

// Status of the last launch on this mesh (device status + failure report);
// throws on failure.  The stream must be synchronised.
static void check_batch(SolverMixed& W, int lpr, int nb, cudaStream_t s) {
    int hst = 0;
    float hdiag[8];
    BT_CUDA(cudaMemcpyAsync(&hst, W.status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    BT_CUDA(cudaMemcpyAsync(hdiag, W.diag.p, sizeof(hdiag), cudaMemcpyDeviceToHost, s));
    BT_CUDA(cudaStreamSynchronize(s));
    if (hst == DEV_NOT_CONVERGED) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "mixed stepper: %s did not converge (step %d, sweep %d, iteration %d, RHS %d at %.3g x its "
                 "target; lanes-per-row %d, %d blocks)",
                 hdiag[0] == 1.0f ? "inner COCG" : "the refinement", (int)hdiag[1], (int)hdiag[2], (int)hdiag[3],
                 (int)hdiag[5], hdiag[4], lpr, nb);
        throw Error(BT_ERR_NOT_CONVERGED, msg);
    }
    map_status_mixed(hst);
}

// Launch one batch (R <= 512 slots) on one mesh with the given geometry.
// Returns the device time of the stepper kernel (ms).
// Launch options of the discrete adjoint: the initial per-signal state (copied
// over the one prepare_batch sets, or zero), per-step saves, the w right-hand
// side of the first step, and a schedule other than the context's (pointers
// already offset to the first step, rows of sched_stride steps).
struct MixExtra {
    const float2* init_h = nullptr;
    const float2* init_l = nullptr;
    bool zero_init = false;
    float2* save_h = nullptr;
    float2* save_l = nullptr;
    int save_every = 1;
    int rhs_w = 0;
    const double* fnew = nullptr;
    const double* fold = nullptr;
};

// Apply the adjoint's launch options to prepared arguments (and the initial state).
static void apply_extra(bt_ctx* ctx, SolverMixed& W, MixArgs& a, const MixExtra* ex) {
    cudaStream_t s = ctx->stream;
    const size_t vsz = (size_t)ctx->mesh.n_dofs * (a.Rp / 2);
    if (ex->zero_init) {
        W.uh.zero(s);
        W.ul.zero(s);
    } else if (ex->init_h) {
        BT_CUDA(cudaMemcpyAsync(W.uh.p, ex->init_h, vsz * sizeof(float2), cudaMemcpyDeviceToDevice, s));
        BT_CUDA(cudaMemcpyAsync(W.ul.p, ex->init_l, vsz * sizeof(float2), cudaMemcpyDeviceToDevice, s));
    }
    a.save_h = ex->save_h;
    a.save_l = ex->save_l;
    a.save_every = std::max(1, ex->save_every);
    a.rhs_w = ex->rhs_w;
    if (ex->fnew) {
        a.fnew = ex->fnew;
        a.fold = ex->fold;
    }
}

static float launch_batch(bt_ctx* ctx, SolverMixed& W, int R, int lpr, int per_sm_blocks, int blocked, int n_steps,
                          double rtol, int maxit, const double* d_u0, const MixExtra* ex = nullptr) {
    cudaStream_t s = ctx->stream;
    const bool extras = ctx->per.on || (ex && (ex->rhs_w || ex->save_h));
    const bool single = !extras && ctx->opt_mixed_inner == 1;
    KFn fn = kernel_for(lpr, extras, single);
    int occ = 0;
    BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kThreadsB, 0));
    BT_REQUIRE(occ >= 1, BT_ERR_CUDA, "mixed stepper kernel does not fit on an SM");
    const int per_sm = std::max(1, std::min(occ, per_sm_blocks));
    const int nb = std::max(1, std::min(per_sm * ctx->num_sms, blocks_needed(ctx, R, lpr)));
    MixArgs a = prepare_batch(ctx, W, R, lpr, nb, blocked, n_steps, rtol, maxit, d_u0, single);
    if (ex) apply_extra(ctx, W, a, ex);
    void* args[] = {&a};
    BT_CUDA(cudaEventRecord(ctx->ev1, s));
    BT_CUDA(cudaLaunchCooperativeKernel((const void*)fn, dim3(nb), dim3(kThreadsB), args, 0, s));
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    check_batch(W, lpr, nb, s);
    float ms = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2));
    return ms;
}

// Measuring autotuner: for this (n, R) try every valid lanes-per-row, 1 and 2
// blocks per SM, and interleaved or blocked row ownership on a 3-step run; keep
// the fastest.  Options fix any of the three.
static SolverMixed::Geo autotune_mixed(bt_ctx* ctx, SolverMixed& W, int R, double rtol, int maxit,
                                       const double* d_u0) {
    const auto key = std::make_pair(ctx->mesh.n_dofs, R);
    auto it = W.tuned.find(key);
    if (it != W.tuned.end()) return it->second;
    std::vector<int> lprs = lpr_candidates(R), bpss = {1, 2}, blks = {0, 1};
    if (ctx->opt_mixed_lpr > 0) lprs = {ctx->opt_mixed_lpr};
    if (ctx->opt_mixed_blocks_per_sm > 0) bpss = {ctx->opt_mixed_blocks_per_sm};
    if (ctx->opt_mixed_blocked >= 0) blks = {ctx->opt_mixed_blocked};
    SolverMixed::Geo best{-1, 1, 0};
    if (lprs.size() * bpss.size() * blks.size() == 1) {
        best = {lprs[0], bpss[0], blks[0]};
    } else {
        float best_ms = 1e30f;
        const int steps = std::min(3, ctx->sched.n_steps);
        for (int lpr : lprs)
            for (int bps : bpss)
                for (int blk : blks) {
                    const float ms = launch_batch(ctx, W, R, lpr, bps, blk, steps, rtol, maxit, d_u0);
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = {lpr, bps, blk};
                    }
                }
    }
    BT_REQUIRE(best.lpr > 0, BT_ERR_INVALID, "mixed stepper: no valid geometry for this batch size");
    W.tuned[key] = best;
    return best;
}

// Packed double-float matrices, row data and the schedule of this mesh.
static SolverMixed& pack_mixed(bt_ctx* ctx, const double* u0, const double** d_u0) {
    Mesh& m = ctx->mesh;
    Assembled& A = ctx->mat;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    if (!ctx->smx) ctx->smx = new SolverMixed();
    SolverMixed& W = *ctx->smx;
    const int64_t nnz = m.nnz;
    W.mA.alloc(nnz);
    W.mL.alloc(nnz);
    W.mS.alloc(nnz);
    W.dg.alloc(m.n_dofs);
    W.w.alloc(m.n_dofs);
    W.rcomp.alloc(m.n_dofs);
    W.iters.alloc(S.n_steps);
    W.sweeps.alloc(S.n_steps);
    k_pack_mixed<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, A.M, A.K, A.T, A.R, A.Jx, A.Jy, A.Jz,
                                                              1.0 / S.dt, S.theta,
                                                              ctx->per.on ? ctx->per.PB.p : nullptr, W.mA, W.mL,
                                                              W.mS);
    BT_CUDA(cudaGetLastError());
    W.fnew.upload(S.f_new.data(), S.f_new.size(), s);
    W.fold.upload(S.f_old.data(), S.f_old.size(), s);
    if (ctx->per.on) {
        BT_REQUIRE(S.phase_set, BT_ERR_STATE, "pseudo-periodic boundaries need bt_set_schedule_phase");
        W.Fint.upload(S.F_old.data(), S.F_old.size(), s);
    }
    if (u0) W.u0.upload(u0, m.n_v, s);
    *d_u0 = u0 ? W.u0.p : nullptr;
    return W;
}

// Slot parameters of NS signals (q, gdir, seq point at the first): slots 2r and
// 2r+1 are Re and Im of signal r; all kMaxRhs slots are filled, the padding with
// copies of the last signal (padding slots start from u = 0 and never iterate).
static void upload_rhs(bt_ctx* ctx, SolverMixed& W, int NS, const double* q, const double* gdir,
                       const int32_t* seq) {
    cudaStream_t s = ctx->stream;
    const int Rmax = kMaxRhs;
    std::vector<double> hq(Rmax);
    std::vector<float> hg(Rmax * 3);
    std::vector<double> hgd(Rmax * 3);
    std::vector<int32_t> hs(Rmax);
    for (int r = 0; r < Rmax; ++r) {
        const int src = std::min(r / 2, NS - 1);
        hq[r] = q[src];
        for (int k = 0; k < 3; ++k) {
            hg[r * 3 + k] = (float)gdir[3 * src + k];
            hgd[r * 3 + k] = gdir[3 * src + k];
        }
        hs[r] = seq ? seq[src] : 0;
        BT_REQUIRE(hs[r] >= 0 && hs[r] < ctx->sched.n_seq, BT_ERR_INVALID, "sequence index out of range");
    }
    W.qv.upload(hq.data(), Rmax, s);
    W.gv.upload(hg.data(), (size_t)Rmax * 3, s);
    W.gvd.upload(hgd.data(), (size_t)Rmax * 3, s);
    W.seqv.upload(hs.data(), Rmax, s);
}

// Signals (sig[0..NS-1], comp_sig optional), per-step iteration counts and, when
// `keep`, the final states of the last launch on this mesh; b0 is the index of
// the batch's first signal among the mesh's signals.
static void collect_batch(bt_ctx* ctx, SolverMixed& W, int b0, int NS, bool keep, double* sig, double* comp_sig,
                          bt_stats* st, const int32_t* orig = nullptr) {
    Mesh& m = ctx->mesh;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    std::vector<int32_t> hit(S.n_steps), hsw(S.n_steps);
    const int Rp = W.Rp;
    std::vector<double> hsig((size_t)Rp * (1 + kMaxCompartments));
    W.sig.download(hsig.data(), hsig.size(), s);
    W.iters.download(hit.data(), S.n_steps, s);
    W.sweeps.download(hsw.data(), S.n_steps, s);
    const int nsr = Rp / 2;   // signals per row in the per-signal arrays
    std::vector<float2> huh(keep ? (size_t)m.n_dofs * nsr : 0), hul(keep ? (size_t)m.n_dofs * nsr : 0);
    if (keep) {
        W.uh.download(huh.data(), huh.size(), s);
        W.ul.download(hul.data(), hul.size(), s);
    }
    BT_CUDA(cudaStreamSynchronize(s));
    // signal r of the batch is signal b0 + r of the call, or orig[b0 + r] when the
    // call's signals were reordered (sig and comp_sig are then the call's arrays)
    for (int r = 0; r < NS; ++r) {
        const size_t so = (size_t)(2 * r) * (1 + kMaxCompartments);   // signal r lives in slot 2r
        const size_t o = orig ? (size_t)orig[b0 + r] : (size_t)(b0 + r);
        const size_t oo = orig ? o : (size_t)r;                        // index into sig / comp_sig
        sig[oo] = hsig[so];
        if (comp_sig)
            for (int c = 0; c < m.n_comp; ++c) comp_sig[oo * m.n_comp + c] = hsig[so + 1 + c];
        for (int64_t i = 0; keep && i < m.n_dofs; ++i) {
            const float2 h = huh[(size_t)i * nsr + r], l = hul[(size_t)i * nsr + r];
            W.saved[o * m.n_dofs + i] = make_double2((double)h.x + l.x, (double)h.y + l.y);
        }
        for (int k = 0; k < S.n_steps; ++k) ctx->last_iters[o * S.n_steps + k] = hit[k];
    }
    if (st) {
        for (int k = 0; k < S.n_steps; ++k) {
            st->max_iterations = std::max(st->max_iterations, hit[k]);
            st->total_iterations += (int64_t)hit[k] * NS;
            st->refinements += hsw[k];
        }
    }
}

static void reset_stats(bt_stats* st, int32_t steps, double rtol) {
    if (!st) return;
    st->steps = steps;
    st->max_iterations = 0;
    st->total_iterations = 0;
    st->max_rel_residual = rtol;
    st->refinements = 0;
    st->graph_launches = 0;
    st->kernel_launches = 0;
    st->stepper_ms = 0.0;
}

// Final states are kept for bt_get_solution only for modest batches (the copy
// is n_dofs x n_signals complex values through the host).
static bool keep_states(bt_ctx* ctx, SolverMixed& W, int32_t nsig) {
    const bool keep = (int64_t)nsig * ctx->mesh.n_dofs <= (int64_t)8 * 1024 * 1024;
    W.saved.assign(keep ? (size_t)nsig * ctx->mesh.n_dofs : 0, make_double2(0.0, 0.0));
    W.saved_nsig = keep ? nsig : 0;
    ctx->last_iters.assign((size_t)nsig * ctx->sched.n_steps, 0);
    return keep;
}

void solve_mixed(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq,
                 const double* u0, double rtol, int32_t maxit, double* sig, double* comp_sig, bt_stats* st) {
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    const double* d_u0 = nullptr;
    SolverMixed& W = pack_mixed(ctx, u0, &d_u0);
    reset_stats(st, S.n_steps, rtol);
    const bool keep = keep_states(ctx, W, nsig);
    // Signals ordered by (sequence, |q|) before they are cut into launches and warps:
    // a launch iterates until its slowest signal converges and a warp of 32 signals
    // until its slowest lane does, and the inner iteration count grows with q f, so
    // signals of similar q share launches and warps (outputs keep the call's order).
    std::vector<int32_t> ord(nsig);
    for (int32_t i = 0; i < nsig; ++i) ord[i] = i;
    if (ctx->opt_mixed_sort)
        std::stable_sort(ord.begin(), ord.end(), [&](int32_t x, int32_t y) {
            const int32_t sx = seq ? seq[x] : 0, sy = seq ? seq[y] : 0;
            if (sx != sy) return sx < sy;
            return std::fabs(q[x]) < std::fabs(q[y]);
        });
    std::vector<double> qo(nsig), go((size_t)nsig * 3);
    std::vector<int32_t> so(seq ? nsig : 0);
    for (int32_t i = 0; i < nsig; ++i) {
        qo[i] = q[ord[i]];
        for (int k = 0; k < 3; ++k) go[(size_t)3 * i + k] = gdir[(size_t)3 * ord[i] + k];
        if (seq) so[i] = seq[ord[i]];
    }
    BT_CUDA(cudaEventRecord(ctx->ev0, s));
    float stepper_ms = 0.0f;
    for (int32_t b0 = 0; b0 < nsig; b0 += kMaxRhs / 2) {
        const int NS = std::min<int32_t>(kMaxRhs / 2, nsig - b0);   // signals in this launch
        const int R = 2 * NS;                                        // slots: Re and Im of each
        upload_rhs(ctx, W, NS, qo.data() + b0, go.data() + 3 * b0, seq ? so.data() + b0 : nullptr);
        const auto geo = autotune_mixed(ctx, W, R, rtol, maxit, d_u0);
        stepper_ms += launch_batch(ctx, W, R, geo.lpr, geo.per_sm, geo.blocked, S.n_steps, rtol, maxit, d_u0);
        collect_batch(ctx, W, b0, NS, keep, sig, comp_sig, st, ord.data());
        if (st) st->kernel_launches += 3;
    }
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    BT_CUDA(cudaEventSynchronize(ctx->ev2));
    float total = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total, ctx->ev0, ctx->ev2));
    if (st) {
        st->gpu_ms = total;
        st->stepper_ms = stepper_ms;
    }
    ctx->last_nsig = nsig;
}

// ---------------------------------------------------------------- several meshes
// Blocks of one cooperative launch shared among meshes in proportion to the
// estimated work of an iteration (matrix + vector bytes), weighted by n^(1/3)
// for the iteration count growing with mesh refinement; every mesh gets at least
// one block and none more than it can use.
static std::vector<int> split_blocks(bt_ctx* const* ctxs, int nm, const std::vector<int>& R, int lpr, int total) {
    BT_REQUIRE(nm <= total, BT_ERR_INVALID, "bt_solve_multi: more meshes than co-resident blocks");
    std::vector<double> w(nm);
    std::vector<int> need(nm), nb(nm);
    double sw = 0.0;
    for (int m = 0; m < nm; ++m) {
        const Mesh& M = ctxs[m]->mesh;
        const int Rp = padded_rhs(R[m], lpr);
        w[m] = (20.0 * (double)M.nnz + 96.0 * (double)M.n_dofs * Rp) * std::cbrt((double)M.n_dofs);
        need[m] = blocks_needed(ctxs[m], R[m], lpr);
        sw += w[m];
    }
    int used = 0;
    for (int m = 0; m < nm; ++m) {
        nb[m] = std::max(1, std::min(need[m], (int)std::floor(total * w[m] / sw)));
        used += nb[m];
    }
    while (used > total) {   // rounding up to one block each can overshoot
        int j = (int)(std::max_element(nb.begin(), nb.end()) - nb.begin());
        if (nb[j] <= 1) break;
        --nb[j];
        --used;
    }
    while (used < total) {   // leftovers to the mesh with the most work per block
        int j = -1;
        double best = 0.0;
        for (int m = 0; m < nm; ++m)
            if (nb[m] < need[m] && w[m] / nb[m] > best) {
                best = w[m] / nb[m];
                j = m;
            }
        if (j < 0) break;
        ++nb[j];
        ++used;
    }
    return nb;
}

// One launch of the multi-mesh kernel; returns its device time (ms).
static float launch_multi(bt_ctx* const* ctxs, int nm, const std::vector<int>& R, int lpr, int n_steps_cap,
                          double rtol, int maxit, const std::vector<const double*>& d_u0,
                          const std::vector<MixExtra>* ex = nullptr) {
    bt_ctx* c0 = ctxs[0];
    cudaStream_t s = c0->stream;
    bool extras = false;
    for (int m = 0; m < nm; ++m)
        extras = extras || ctxs[m]->per.on || (ex && ((*ex)[m].rhs_w || (*ex)[m].save_h));
    const bool single = !extras && c0->opt_mixed_inner == 1;
    KFnMulti fn = kernel_multi_for(lpr, extras, single);
    int occ = 0;
    BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kThreadsB, 0));
    BT_REQUIRE(occ >= 1, BT_ERR_CUDA, "mixed stepper kernel does not fit on an SM");
    const int per_sm =
        c0->opt_mixed_blocks_per_sm > 0 ? std::min(occ, c0->opt_mixed_blocks_per_sm) : std::min(occ, 2);
    const int total = per_sm * c0->num_sms;
    const std::vector<int> nb = split_blocks(ctxs, nm, R, lpr, total);
    std::vector<MixArgs> args(nm);
    std::vector<int> first(nm + 1, 0);
    for (int m = 0; m < nm; ++m) {
        SolverMixed& W = *ctxs[m]->smx;
        const int steps = std::min(n_steps_cap, ctxs[m]->sched.n_steps);
        args[m] = prepare_batch(ctxs[m], W, R[m], lpr, nb[m], 0, steps, rtol, maxit, d_u0[m], single);
        if (ex) apply_extra(ctxs[m], W, args[m], &(*ex)[m]);
        first[m + 1] = first[m] + nb[m];
    }
    SolverMixed& W0 = *c0->smx;
    W0.margs.upload(args.data(), nm, s);
    W0.mfirst.upload(first.data(), nm + 1, s);
    const MixArgs* pa = W0.margs.p;
    const int* pf = W0.mfirst.p;
    int nmi = nm;
    void* kargs[] = {&pa, &pf, &nmi};
    BT_CUDA(cudaEventRecord(c0->ev1, s));
    BT_CUDA(cudaLaunchCooperativeKernel((const void*)fn, dim3(first[nm]), dim3(kThreadsB), kargs, 0, s));
    BT_CUDA(cudaEventRecord(c0->ev2, s));
    for (int m = 0; m < nm; ++m) check_batch(*ctxs[m]->smx, lpr, nb[m], s);
    float ms = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&ms, c0->ev1, c0->ev2));
    return ms;
}

// Meshes that cannot fill the GPU alone, in one persistent launch (all on the
// first context's stream).
static void multi_launch_group(bt_ctx* const* ctxs, int32_t nm, const int32_t* nsig, const double* q,
                               const double* gdir, const int32_t* seq, double rtol, int32_t maxit, double* sig,
                               bt_stats* st) {
    bt_ctx* c0 = ctxs[0];
    cudaStream_t s = c0->stream;
    std::vector<int> R(nm);
    std::vector<const double*> d_u0(nm, nullptr);
    std::vector<int64_t> off(nm + 1, 0);
    std::vector<char> keep(nm);
    int32_t steps = 0;
    for (int m = 0; m < nm; ++m) {
        off[m + 1] = off[m] + nsig[m];
        R[m] = 2 * nsig[m];
        SolverMixed& W = pack_mixed(ctxs[m], nullptr, &d_u0[m]);
        upload_rhs(ctxs[m], W, nsig[m], q + off[m], gdir + 3 * off[m], seq ? seq + off[m] : nullptr);
        keep[m] = keep_states(ctxs[m], W, nsig[m]);
        steps = std::max(steps, ctxs[m]->sched.n_steps);
    }
    reset_stats(st, steps, rtol);
    // a lanes-per-row every mesh's batch can use (small batches are padded to
    // the chunk), chosen on 3-step runs
    std::vector<int> cands;
    for (int lpr = 1; lpr <= 32; lpr <<= 1) {
        bool ok = true;
        for (int m = 0; m < nm; ++m) ok = ok && padded_rhs(R[m], lpr) > 0;
        if (ok) cands.push_back(lpr);
    }
    if (c0->opt_mixed_lpr > 0) cands = {c0->opt_mixed_lpr};
    BT_REQUIRE(!cands.empty(), BT_ERR_INVALID, "bt_solve_multi: no lanes-per-row fits every mesh's batch");
    int lpr = cands[0];
    // the choice is cached per set of (mesh size, batch size), so repeated calls of
    // the same problem run the same geometry and give bitwise the same signals
    std::vector<int64_t> key;
    for (int m = 0; m < nm; ++m) {
        key.push_back(ctxs[m]->mesh.n_dofs);
        key.push_back(R[m]);
    }
    SolverMixed& Wc = *c0->smx;
    auto hit = Wc.tuned_multi.find(key);
    if (c0->opt_mixed_lpr <= 0 && hit != Wc.tuned_multi.end()) {
        lpr = hit->second;
    } else if (cands.size() > 1) {
        float best = 1e30f;
        for (int c : cands) {
            const float ms = launch_multi(ctxs, nm, R, c, 3, rtol, maxit, d_u0);
            if (ms < best) {
                best = ms;
                lpr = c;
            }
        }
        Wc.tuned_multi[key] = lpr;
    }
    BT_CUDA(cudaEventRecord(c0->ev0, s));
    const float ms = launch_multi(ctxs, nm, R, lpr, 1 << 30, rtol, maxit, d_u0);
    for (int m = 0; m < nm; ++m) {
        collect_batch(ctxs[m], *ctxs[m]->smx, 0, nsig[m], keep[m] != 0, sig + off[m], nullptr, st);
        ctxs[m]->last_nsig = nsig[m];
    }
    BT_CUDA(cudaEventRecord(c0->ev2, s));
    BT_CUDA(cudaEventSynchronize(c0->ev2));
    float total = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total, c0->ev0, c0->ev2));
    if (st) {
        st->gpu_ms = total;
        st->stepper_ms = ms;
        st->kernel_launches = 2 * nm + 1;
    }
}

static void add_stats(bt_stats* st, const bt_stats& a) {
    if (!st) return;
    st->steps = std::max(st->steps, a.steps);
    st->max_iterations = std::max(st->max_iterations, a.max_iterations);
    st->total_iterations += a.total_iterations;
    st->refinements += a.refinements;
    st->kernel_launches += a.kernel_launches;
    st->stepper_ms += a.stepper_ms;
    st->gpu_ms += a.gpu_ms;
}

// Several meshes: a mesh whose batch fills every co-resident block slot by itself
// (two blocks of 8 warp-units per SM) runs alone on the whole GPU, back to back
// with the other large ones; the remaining small meshes share one persistent
// launch, one sub-grid each (a large mesh gains nothing from sharing the GPU's
// blocks and would lose most of them).
void solve_mixed_multi(bt_ctx* const* ctxs, int32_t nm, const int32_t* nsig, const double* q, const double* gdir,
                       const int32_t* seq, double rtol, int32_t maxit, double* sig, bt_stats* st) {
    bt_ctx* c0 = ctxs[0];
    cudaStream_t s = c0->stream;
    // every mesh's work goes on the first context's stream for this call
    std::vector<cudaStream_t> saved(nm);
    for (int m = 0; m < nm; ++m) {
        BT_CUDA(cudaStreamSynchronize(ctxs[m]->stream));
        saved[m] = ctxs[m]->stream;
        ctxs[m]->stream = s;
    }
    struct Restore {
        bt_ctx* const* c;
        std::vector<cudaStream_t>& v;
        ~Restore() {
            for (size_t m = 0; m < v.size(); ++m) c[m]->stream = v[m];
        }
    } restore{ctxs, saved};
    std::vector<int64_t> off(nm + 1, 0);
    for (int m = 0; m < nm; ++m) off[m + 1] = off[m] + nsig[m];
    std::vector<int> small, large;
    for (int m = 0; m < nm; ++m) {
        // warp-units of the batch: rows x slots / 64, whatever the lanes-per-row
        const int64_t units = ctxs[m]->mesh.n_dofs * (int64_t)ceil_pow2(2 * nsig[m]) / 64;
        (units / kWarpsB >= 2 * ctxs[m]->num_sms ? large : small).push_back(m);
    }
    if (small.size() == 1) {
        large.push_back(small[0]);
        small.clear();
    }
    reset_stats(st, 0, rtol);
    BT_CUDA(cudaEventRecord(c0->ev3, s));
    for (int m : large) {
        bt_stats one{};
        solve_mixed(ctxs[m], nsig[m], q + off[m], gdir + 3 * off[m], seq ? seq + off[m] : nullptr, nullptr, rtol,
                    maxit, sig + off[m], nullptr, &one);
        add_stats(st, one);
    }
    if (!small.empty()) {
        std::vector<bt_ctx*> cs;
        std::vector<int32_t> ns;
        std::vector<double> qs, gs, out;
        std::vector<int32_t> ss;
        for (int m : small) {
            cs.push_back(ctxs[m]);
            ns.push_back(nsig[m]);
            qs.insert(qs.end(), q + off[m], q + off[m + 1]);
            gs.insert(gs.end(), gdir + 3 * off[m], gdir + 3 * off[m + 1]);
            if (seq) ss.insert(ss.end(), seq + off[m], seq + off[m + 1]);
        }
        out.resize(qs.size());
        bt_stats grp{};
        multi_launch_group(cs.data(), (int32_t)cs.size(), ns.data(), qs.data(), gs.data(), seq ? ss.data() : nullptr,
                           rtol, maxit, out.data(), &grp);
        add_stats(st, grp);
        size_t k = 0;
        for (int m : small)
            for (int32_t i = 0; i < nsig[m]; ++i) sig[off[m] + i] = out[k++];
    }
    BT_CUDA(cudaEventRecord(c0->ev2, s));
    BT_CUDA(cudaEventSynchronize(c0->ev2));
    float total = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total, c0->ev3, c0->ev2));
    if (st) st->gpu_ms = total;
}

void get_solution_mixed(bt_ctx* ctx, int32_t index, double* u) {
    BT_REQUIRE(ctx->smx && index >= 0 && index < ctx->smx->saved_nsig, BT_ERR_INVALID,
               "bt_get_solution: no such signal in the last mixed solve (states of batches above "
               "8M dof-signals are not kept)");
    const int64_t n = ctx->mesh.n_dofs;
    const double2* src = ctx->smx->saved.data() + (size_t)index * n;
    for (int64_t i = 0; i < n; ++i) {
        u[2 * i] = src[i].x;
        u[2 * i + 1] = src[i].y;
    }
}

void reset_tuning_mixed(bt_ctx* ctx) {
    if (ctx->smx) {
        ctx->smx->tuned.clear();
        ctx->smx->tuned_multi.clear();
    }
}

void free_solver_mixed(bt_ctx* ctx) {
    delete ctx->smx;
    ctx->smx = nullptr;
}

// ------------------------------------------------------- batched discrete adjoint
// The FP64 adjoint of stepper64.cu (adjoint_fp64) for a whole batch of signals in
// mixed precision: with A_n u_{n+1} = B_n u_n and Sig = w^T Re(u_N),
//     A_{N-1} lambda_N = w,   A_{n-1} lambda_n = B_n lambda_{n+1}  (A, B complex symmetric),
//     dSig/dxi = -Re sum_n lambda_{n+1}^T (dS/dxi) (theta u_{n+1} + (1 - theta) u_n).
// A backward step is a forward step of the batched stepper with the schedule
// pair (f_new[n-1], f_old[n]), so the same kernel runs both directions; forward
// states are recomputed segment by segment from checkpoints every stride steps.
namespace {

// per-cell geometry: the gradients G_1..G_3 of the barycentric coordinates of
// vertices 1..3 (G_0 = -(G_1 + G_2 + G_3)) and the volume, as 12 floats
__global__ void k_cell_grad(int64_t n_t, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                            float4* __restrict__ geo) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_t) return;
    double X[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) X[k][c] = xyz[(int64_t)tets[t * 4 + k] * 3 + c];
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
    const double g[9] = {c00 * id, c01 * id, c02 * id,
                         (E[0][2] * E[2][1] - E[0][1] * E[2][2]) * id,
                         (E[0][0] * E[2][2] - E[0][2] * E[2][0]) * id,
                         (E[0][1] * E[2][0] - E[0][0] * E[2][1]) * id,
                         (E[0][1] * E[1][2] - E[0][2] * E[1][1]) * id,
                         (E[0][2] * E[1][0] - E[0][0] * E[1][2]) * id,
                         (E[0][0] * E[1][1] - E[0][1] * E[1][0]) * id};
    geo[t * 3 + 0] = make_float4((float)g[0], (float)g[1], (float)g[2], (float)g[3]);
    geo[t * 3 + 1] = make_float4((float)g[4], (float)g[5], (float)g[6], (float)g[7]);
    geo[t * 3 + 2] = make_float4((float)g[8], (float)(fabs(det) / 6.0), 0.0f, 0.0f);
}

// x_k - x_0 of a double-float (hi, lo) state: the hi parts of nearby values
// subtract exactly, the lo parts restore the digits the difference needs
__device__ __forceinline__ float2 df_diff(const float2* __restrict__ h, const float2* __restrict__ l, size_t ik,
                                          size_t i0) {
    const float2 hk = h[ik], h0 = h[i0], lk = l[ik], l0 = l[i0];
    return make_float2((hk.x - h0.x) + (lk.x - l0.x), (hk.y - h0.y) + (lk.y - l0.y));
}

// accD[t][s] -= Re(L^T K V), accT[t][s] -= Re(L^T M V) of cell t, signal s (unit
// coefficients).  L^T K V = vol grad(L) . grad(V) with the gradients formed from
// vertex differences (the rows of K sum to zero, so products of the raw vertex
// values would cancel); M = vol/20 (1 + delta_rc).  FP32 products, FP64 sums.
__global__ void k_adjb_cells(int64_t n_t, int NS, int ns, const float4* __restrict__ geo,
                             const int32_t* __restrict__ tets, const int32_t* __restrict__ comp,
                             const int32_t* __restrict__ dof_of, int nc, const float2* __restrict__ lh,
                             const float2* __restrict__ ll, const float2* __restrict__ u0h,
                             const float2* __restrict__ u0l, const float2* __restrict__ u1h,
                             const float2* __restrict__ u1l, double theta, double* __restrict__ accD,
                             double* __restrict__ accT) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_t * NS) return;
    const int64_t t = idx / NS;
    const int sg = (int)(idx % NS);
    const int f = comp[t];
    size_t i[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) i[k] = (size_t)dof_of[(int64_t)tets[t * 4 + k] * nc + f] * ns + sg;
    const float th = (float)theta, om = (float)(1.0 - theta);
    const float4 a = geo[t * 3 + 0], b = geo[t * 3 + 1], c = geo[t * 3 + 2];
    const float G[3][3] = {{a.x, a.y, a.z}, {a.w, b.x, b.y}, {b.z, b.w, c.x}};
    const float vol = c.y;
    float2 gl[3], gv[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) gl[d] = gv[d] = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        const float2 dl = df_diff(lh, ll, i[k], i[0]);
        const float2 d0 = df_diff(u0h, u0l, i[k], i[0]), d1 = df_diff(u1h, u1l, i[k], i[0]);
        const float2 dv = make_float2(th * d1.x + om * d0.x, th * d1.y + om * d0.y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            gl[d].x = fmaf(dl.x, G[k - 1][d], gl[d].x);
            gl[d].y = fmaf(dl.y, G[k - 1][d], gl[d].y);
            gv[d].x = fmaf(dv.x, G[k - 1][d], gv[d].x);
            gv[d].y = fmaf(dv.y, G[k - 1][d], gv[d].y);
        }
    }
    float sK = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) sK += gl[d].x * gv[d].x - gl[d].y * gv[d].y;
    float2 sl = make_float2(0.f, 0.f), sv = sl;
    float sd = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 L = lh[i[k]], A0 = u0h[i[k]], A1 = u1h[i[k]];
        const float2 V = make_float2(th * A1.x + om * A0.x, th * A1.y + om * A0.y);
        sl.x += L.x; sl.y += L.y;
        sv.x += V.x; sv.y += V.y;
        sd += L.x * V.x - L.y * V.y;
    }
    const float sM = (vol / 20.0f) * (sl.x * sv.x - sl.y * sv.y + sd);
    accD[idx] -= (double)(vol * sK);
    accT[idx] -= (double)sM;
}

// Per-cell gradients of a weighted sum of the batch's signals, sum_s w_s S_s: one
// warp per cell, lanes over signals, the contraction of k_adjb_cells split into
// the six stored tensor components (xx, yy, zz, xy, xz, yz; an off-diagonal one
// counts D_kl and D_lk) and the mass term; the lanes' sums are added in a fixed
// order (warp tree), so the result is deterministic.
__global__ void k_adjb_cells_w(int64_t n_t, int NS, int ns, const float4* __restrict__ geo,
                               const int32_t* __restrict__ tets, const int32_t* __restrict__ comp,
                               const int32_t* __restrict__ dof_of, int nc, const float2* __restrict__ lh,
                               const float2* __restrict__ ll, const float2* __restrict__ u0h,
                               const float2* __restrict__ u0l, const float2* __restrict__ u1h,
                               const float2* __restrict__ u1l, double theta, const double* __restrict__ wsig,
                               double* __restrict__ acc6, double* __restrict__ accT) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float th = (float)theta, om = (float)(1.0 - theta);
    for (int64_t t = warp; t < n_t; t += nwarps) {
        const int f = comp[t];
        size_t base[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) base[k] = (size_t)dof_of[(int64_t)tets[t * 4 + k] * nc + f] * ns;
        const float4 a = geo[t * 3 + 0], b = geo[t * 3 + 1], c = geo[t * 3 + 2];
        const float G[3][3] = {{a.x, a.y, a.z}, {a.w, b.x, b.y}, {b.z, b.w, c.x}};
        const double vol = (double)c.y;
        double o[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int sg = lane; sg < NS; sg += 32) {
            float2 gl[3], gv[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) gl[d] = gv[d] = make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 1; k < 4; ++k) {
                const float2 dl = df_diff(lh, ll, base[k] + sg, base[0] + sg);
                const float2 d0 = df_diff(u0h, u0l, base[k] + sg, base[0] + sg),
                             d1 = df_diff(u1h, u1l, base[k] + sg, base[0] + sg);
                const float2 dv = make_float2(th * d1.x + om * d0.x, th * d1.y + om * d0.y);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    gl[d].x = fmaf(dl.x, G[k - 1][d], gl[d].x);
                    gl[d].y = fmaf(dl.y, G[k - 1][d], gl[d].y);
                    gv[d].x = fmaf(dv.x, G[k - 1][d], gv[d].x);
                    gv[d].y = fmaf(dv.y, G[k - 1][d], gv[d].y);
                }
            }
            auto re = [&](int k, int l) { return gl[k].x * gv[l].x - gl[k].y * gv[l].y; };
            float2 sl = make_float2(0.f, 0.f), sv = sl;
            float sd = 0.f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 L = lh[base[k] + sg], A0 = u0h[base[k] + sg], A1 = u1h[base[k] + sg];
                const float2 V = make_float2(th * A1.x + om * A0.x, th * A1.y + om * A0.y);
                sl.x += L.x; sl.y += L.y;
                sv.x += V.x; sv.y += V.y;
                sd += L.x * V.x - L.y * V.y;
            }
            const double w = wsig[sg];
            o[0] += w * (double)re(0, 0);
            o[1] += w * (double)re(1, 1);
            o[2] += w * (double)re(2, 2);
            o[3] += w * (double)(re(0, 1) + re(1, 0));
            o[4] += w * (double)(re(0, 2) + re(2, 0));
            o[5] += w * (double)(re(1, 2) + re(2, 1));
            o[6] += w * (double)(sl.x * sv.x - sl.y * sv.y + sd);
        }
#pragma unroll
        for (int k = 0; k < 7; ++k) o[k] = warp_sum(o[k]);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 6; ++k) acc6[t * 6 + k] -= vol * o[k];
            accT[t] -= vol / 20.0 * o[6];
        }
    }
}

__device__ __forceinline__ double2 state_at(const float2* __restrict__ h, const float2* __restrict__ l, size_t i) {
    const float2 a = h[i], b = l[i];
    return make_double2((double)a.x + (double)b.x, (double)a.y + (double)b.y);
}

// accK[i][s] -= Re([L]^T B [V]) of interface facet i (facet mass, jumps across the duplicated dofs)
__global__ void k_adjb_facets(int64_t n_if, int NS, int ns, const int32_t* __restrict__ fcell,
                              const int32_t* __restrict__ fface, const double* __restrict__ xyz,
                              const int32_t* __restrict__ tets, const int32_t* __restrict__ nbr,
                              const int32_t* __restrict__ comp, const int32_t* __restrict__ dof_of, int nc,
                              const float2* __restrict__ lh, const float2* __restrict__ ll,
                              const float2* __restrict__ u0h, const float2* __restrict__ u0l,
                              const float2* __restrict__ u1h, const float2* __restrict__ u1l, double theta,
                              double* __restrict__ accK) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_if * NS) return;
    const int64_t i = idx / NS;
    const int sg = (int)(idx % NS);
    const int32_t t = fcell[i];
    const int fa = fface[i];
    const int32_t nb = nbr[(int64_t)t * 4 + fa];
    const int f = comp[t], g = comp[nb];
    int32_t fv[3];
    int m = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k != fa) fv[m++] = tets[(int64_t)t * 4 + k];
    double e1[3], e2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        e1[c] = xyz[(int64_t)fv[1] * 3 + c] - xyz[(int64_t)fv[0] * 3 + c];
        e2[c] = xyz[(int64_t)fv[2] * 3 + c] - xyz[(int64_t)fv[0] * 3 + c];
    }
    const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                 cz = e1[0] * e2[1] - e1[1] * e2[0];
    const double area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
    double2 Lj[3], Vj[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const size_t da = (size_t)dof_of[(int64_t)fv[k] * nc + f] * ns + sg;
        const size_t db = (size_t)dof_of[(int64_t)fv[k] * nc + g] * ns + sg;
        const double2 la = state_at(lh, ll, da), lb = state_at(lh, ll, db);
        const double2 ua0 = state_at(u0h, u0l, da), ua1 = state_at(u1h, u1l, da);
        const double2 ub0 = state_at(u0h, u0l, db), ub1 = state_at(u1h, u1l, db);
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
    accK[idx] -= sK;
}

// out[s][k] = sum over items i with key[i] == k of acc[i][s], in a fixed order
// (grid: NS x n_keys blocks of 256 threads)
__global__ void k_adjb_reduce(int64_t n_items, int NS, const int32_t* __restrict__ key, int n_keys,
                              const double* __restrict__ acc, double* __restrict__ out) {
    __shared__ double sm[256];
    const int sg = blockIdx.x, kk = blockIdx.y;
    double v = 0.0;
    for (int64_t i = threadIdx.x; i < n_items; i += blockDim.x)
        if (key[i] == kk) v += acc[i * NS + sg];
    sm[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)sg * n_keys + kk] = sm[0];
}

}  // namespace

// One mesh's part of the batched adjoint: its adjoint schedule, cell gradients,
// interface-facet -> region-pair map, and the per-batch checkpoint, segment,
// backward-state and accumulator buffers.
struct AdjMesh {
    bt_ctx* ctx = nullptr;
    SolverMixed* W = nullptr;
    const double* d_u0 = nullptr;
    int NS = 0, R = 0, Rp = 0, ns = 0;
    size_t vsz = 0;
    DevBuf<double> afn, afo, accD, accT, accK, red;
    DevBuf<float4> cgeo;
    DevBuf<int32_t> pair;
    DevBuf<float2> ckh, ckl, sgh, sgl, bkh, bkl, lch, lcl;
    // per-cell gradients of a weighted signal sum (nullable): weights of the
    // batch's signals, accumulators over all batches
    DevBuf<double> wsig;
    double* acc6 = nullptr;
    double* accTc = nullptr;
};

static void adj_mesh_setup(AdjMesh& A, bt_ctx* ctx, bool cells = false) {
    Mesh& m = ctx->mesh;
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    BT_REQUIRE(cells || (!ctx->coeffs.has_cell_D && !ctx->coeffs.has_cell_T2), BT_ERR_STATE,
               "batched adjoint: per-region gradients need per-region coefficients (clear per-cell D / T2, or use "
               "bt_adjoint_batch_cells)");
    BT_REQUIRE(!ctx->per.on, BT_ERR_STATE, "batched adjoint: not defined with pseudo-periodic boundaries");
    BT_REQUIRE(!ctx->coeffs.kappa_cr, BT_ERR_STATE,
               "batched adjoint: gradients are defined for one permeability per facet (not the Crouzeix-Raviart mode)");
    A.ctx = ctx;
    A.W = &pack_mixed(ctx, nullptr, &A.d_u0);
    const int N = S.n_steps, nr = m.n_regions;
    // adjoint schedule: backward step j builds lambda_{N-j} with f_new[N-1-j] and f_old[N-j]
    std::vector<double> afn((size_t)S.n_seq * N), afo((size_t)S.n_seq * N, 0.0);
    for (int r = 0; r < S.n_seq; ++r)
        for (int j = 0; j < N; ++j) {
            afn[(size_t)r * N + j] = S.f_new[(size_t)r * N + N - 1 - j];
            if (j >= 1) afo[(size_t)r * N + j] = S.f_old[(size_t)r * N + N - j];
        }
    A.afn.upload(afn.data(), afn.size(), s);
    A.afo.upload(afo.data(), afo.size(), s);
    A.cgeo.alloc((size_t)m.n_t * 3);
    k_cell_grad<<<(unsigned)((m.n_t + 127) / 128), 128, 0, s>>>(m.n_t, m.xyz, m.tets, A.cgeo);
    BT_CUDA(cudaGetLastError());
    // interface facet -> region pair (r1 <= r2) index r1 * nr + r2
    std::vector<int32_t> hreg(m.n_t), hpair(std::max<int64_t>(1, m.n_iface), 0);
    m.region.download(hreg.data(), m.n_t, s);
    if (m.n_iface > 0) {
        std::vector<int32_t> hfc(m.n_iface), hff(m.n_iface), hnb((size_t)m.n_t * 4);
        m.iface_cell.download(hfc.data(), m.n_iface, s);
        m.iface_face.download(hff.data(), m.n_iface, s);
        m.nbr.download(hnb.data(), hnb.size(), s);
        BT_CUDA(cudaStreamSynchronize(s));
        for (int64_t i = 0; i < m.n_iface; ++i) {
            const int32_t t = hfc[i], nb = hnb[(size_t)t * 4 + hff[i]];
            hpair[i] = std::min(hreg[t], hreg[nb]) * nr + std::max(hreg[t], hreg[nb]);
        }
    }
    A.pair.upload(hpair.data(), hpair.size(), s);
}

// Buffers of one batch of NS signals padded to Rp slots, and checkpoint 0 (u0 = 1).
static void adj_batch_alloc(AdjMesh& A, int NS, int Rp, int nck, int stride) {
    Mesh& m = A.ctx->mesh;
    cudaStream_t s = A.ctx->stream;
    SolverMixed& W = *A.W;
    A.NS = NS;
    A.R = 2 * NS;
    A.Rp = Rp;
    A.ns = Rp / 2;
    A.vsz = (size_t)m.n_dofs * A.ns;
    const size_t vsz = A.vsz;
    A.ckh.alloc((nck + 1) * vsz); A.ckl.alloc((nck + 1) * vsz);
    A.sgh.alloc((stride + 1) * vsz); A.sgl.alloc((stride + 1) * vsz);
    A.bkh.alloc(stride * vsz); A.bkl.alloc(stride * vsz);
    A.lch.alloc(vsz); A.lcl.alloc(vsz);
    A.accD.alloc((size_t)m.n_t * NS); A.accD.zero(s);
    A.accT.alloc((size_t)m.n_t * NS); A.accT.zero(s);
    A.accK.alloc((size_t)std::max<int64_t>(1, m.n_iface) * NS); A.accK.zero(s);
    k_rows_mixed<<<(unsigned)((m.n_dofs + 255) / 256), 256, 0, s>>>(m.n_dofs, Rp, A.R, m.diag_pos, W.mA, A.ctx->mat.w,
                                                                    m.dof_comp, m.dof_vertex, nullptr, W.dg, W.w,
                                                                    W.rcomp, A.ckh.p, A.ckl.p);
    BT_CUDA(cudaGetLastError());
}

// Contractions of backward step n of one mesh (states u_n, u_{n+1} of the segment
// starting at a0, lambda_{n+1}).
static void adj_contract(AdjMesh& A, int n, int a0, int e0, double theta) {
    Mesh& m = A.ctx->mesh;
    cudaStream_t s = A.ctx->stream;
    const size_t vsz = A.vsz;
    const float2* Lh = (n + 1 == e0) ? A.lch.p : A.bkh.p + (size_t)(e0 - 2 - n) * vsz;
    const float2* Ll = (n + 1 == e0) ? A.lcl.p : A.bkl.p + (size_t)(e0 - 2 - n) * vsz;
    const size_t o0 = (size_t)(n - a0) * vsz, o1 = o0 + vsz;
    const unsigned cb = (unsigned)((m.n_t * A.NS + 255) / 256), fb = (unsigned)((m.n_iface * A.NS + 255) / 256);
    k_adjb_cells<<<cb, 256, 0, s>>>(m.n_t, A.NS, A.ns, A.cgeo, m.tets, m.comp, m.dof_of, m.n_comp, Lh, Ll,
                                    A.sgh.p + o0, A.sgl.p + o0, A.sgh.p + o1, A.sgl.p + o1, theta, A.accD, A.accT);
    if (m.n_iface > 0)
        k_adjb_facets<<<fb, 256, 0, s>>>(m.n_iface, A.NS, A.ns, m.iface_cell, m.iface_face, m.xyz, m.tets, m.nbr,
                                         m.comp, m.dof_of, m.n_comp, Lh, Ll, A.sgh.p + o0, A.sgl.p + o0,
                                         A.sgh.p + o1, A.sgl.p + o1, theta, A.accK);
    if (A.acc6) {
        const unsigned wb = (unsigned)std::min<int64_t>((m.n_t + 7) / 8, (int64_t)A.ctx->num_sms * 64);
        k_adjb_cells_w<<<wb, 256, 0, s>>>(m.n_t, A.NS, A.ns, A.cgeo, m.tets, m.comp, m.dof_of, m.n_comp, Lh, Ll,
                                          A.sgh.p + o0, A.sgl.p + o0, A.sgh.p + o1, A.sgl.p + o1, theta, A.wsig,
                                          A.acc6, A.accTc);
    }
    BT_CUDA(cudaGetLastError());
}

// Per-signal sums over regions and region pairs (fixed order) into the outputs of
// signals [b0, b0 + NS) of this mesh.
static void adj_finish(AdjMesh& A, int b0, double* dD, double* dinvT2, double* dkappa) {
    Mesh& m = A.ctx->mesh;
    cudaStream_t s = A.ctx->stream;
    const int NS = A.NS, nr = m.n_regions;
    A.red.alloc((size_t)NS * (2 * nr + nr * nr));
    k_adjb_reduce<<<dim3(NS, nr), 256, 0, s>>>(m.n_t, NS, m.region, nr, A.accD, A.red.p);
    k_adjb_reduce<<<dim3(NS, nr), 256, 0, s>>>(m.n_t, NS, m.region, nr, A.accT, A.red.p + (size_t)NS * nr);
    if (m.n_iface > 0)
        k_adjb_reduce<<<dim3(NS, nr * nr), 256, 0, s>>>(m.n_iface, NS, A.pair, nr * nr, A.accK,
                                                       A.red.p + (size_t)2 * NS * nr);
    BT_CUDA(cudaGetLastError());
    std::vector<double> hr((size_t)NS * (2 * nr + nr * nr), 0.0);
    A.red.download(hr.data(), (size_t)NS * (2 * nr + (m.n_iface > 0 ? nr * nr : 0)), s);
    BT_CUDA(cudaStreamSynchronize(s));
    for (int sg = 0; sg < NS; ++sg) {
        const size_t o = (size_t)(b0 + sg);
        for (int r = 0; r < nr; ++r) {
            if (dD) dD[o * nr + r] = hr[(size_t)sg * nr + r];
            if (dinvT2) dinvT2[o * nr + r] = hr[(size_t)NS * nr + (size_t)sg * nr + r];
        }
        if (dkappa)
            for (int r1 = 0; r1 < nr; ++r1)
                for (int r2 = 0; r2 < nr; ++r2) {
                    const int a = std::min(r1, r2), b = std::max(r1, r2);
                    dkappa[o * nr * nr + (size_t)r1 * nr + r2] =
                        (a == b) ? 0.0 : hr[(size_t)2 * NS * nr + (size_t)sg * nr * nr + (size_t)a * nr + b];
                }
    }
}

// The adjoint pipeline of a group of meshes (one batch each) whose launches are
// shared: launch(n_steps, ex) runs one launch of every mesh in the group with the
// per-mesh extras ex[g] and returns its device time.  All meshes have N steps.
template <typename Launch>
static void adj_pipeline(std::vector<AdjMesh*>& G, int N, int stride, double theta, Launch&& launch,
                         const std::vector<int>& b0, const std::vector<double*>& sig, float& ms,
                         int64_t& launches) {
    const int ng = (int)G.size();
    const int nck = (N + stride - 1) / stride;
    std::vector<MixExtra> ex(ng);
    {   // forward: u_{j stride} into checkpoint j, and the signals
        for (int g = 0; g < ng; ++g) {
            ex[g] = MixExtra();
            ex[g].save_h = G[g]->ckh.p + G[g]->vsz;
            ex[g].save_l = G[g]->ckl.p + G[g]->vsz;
            ex[g].save_every = stride;
        }
        ms += launch(N, ex);
        ++launches;
        for (int g = 0; g < ng; ++g)
            collect_batch(G[g]->ctx, *G[g]->W, b0[g], G[g]->NS, false, sig[g] + b0[g], nullptr, nullptr);
    }
    {   // lambda_N = A_{N-1}^{-1} w from the zero state
        for (int g = 0; g < ng; ++g) {
            ex[g] = MixExtra();
            ex[g].zero_init = true;
            ex[g].rhs_w = 1;
            ex[g].fnew = G[g]->afn.p;
            ex[g].fold = G[g]->afo.p;
        }
        ms += launch(1, ex);
        ++launches;
        for (int g = 0; g < ng; ++g) {
            AdjMesh& A = *G[g];
            cudaStream_t s = A.ctx->stream;
            BT_CUDA(cudaMemcpyAsync(A.lch.p, A.W->uh.p, A.vsz * sizeof(float2), cudaMemcpyDeviceToDevice, s));
            BT_CUDA(cudaMemcpyAsync(A.lcl.p, A.W->ul.p, A.vsz * sizeof(float2), cudaMemcpyDeviceToDevice, s));
        }
    }
    for (int sgm = nck - 1; sgm >= 0; --sgm) {
        const int a0 = sgm * stride, e0 = std::min(a0 + stride, N), len = e0 - a0;
        for (int g = 0; g < ng; ++g) {   // u_{a0..e0}: seg[k] = u_{a0+k}
            AdjMesh& A = *G[g];
            cudaStream_t s = A.ctx->stream;
            BT_CUDA(cudaMemcpyAsync(A.sgh.p, A.ckh.p + (size_t)sgm * A.vsz, A.vsz * sizeof(float2),
                                    cudaMemcpyDeviceToDevice, s));
            BT_CUDA(cudaMemcpyAsync(A.sgl.p, A.ckl.p + (size_t)sgm * A.vsz, A.vsz * sizeof(float2),
                                    cudaMemcpyDeviceToDevice, s));
            ex[g] = MixExtra();
            ex[g].init_h = A.sgh.p;
            ex[g].init_l = A.sgl.p;
            ex[g].save_h = A.sgh.p + A.vsz;
            ex[g].save_l = A.sgl.p + A.vsz;
            ex[g].fnew = A.W->fnew.p + a0;
            ex[g].fold = A.W->fold.p + a0;
        }
        ms += launch(len, ex);
        ++launches;
        // lambda_{e0-1} ... lambda_{a0} (lambda_0 is not needed): bk[k] = lambda_{e0-1-k}
        const int nb_steps = (a0 == 0) ? len - 1 : len;
        if (nb_steps > 0) {
            for (int g = 0; g < ng; ++g) {
                AdjMesh& A = *G[g];
                ex[g] = MixExtra();
                ex[g].init_h = A.lch.p;
                ex[g].init_l = A.lcl.p;
                ex[g].save_h = A.bkh.p;
                ex[g].save_l = A.bkl.p;
                ex[g].fnew = A.afn.p + (N - e0 + 1);
                ex[g].fold = A.afo.p + (N - e0 + 1);
            }
            ms += launch(nb_steps, ex);
            ++launches;
        }
        for (int g = 0; g < ng; ++g) {
            AdjMesh& A = *G[g];
            for (int n = e0 - 1; n >= a0; --n) {
                adj_contract(A, n, a0, e0, theta);
                launches += 1 + (A.ctx->mesh.n_iface > 0);
            }
            if (a0 > 0) {   // lambda_{a0} starts the previous segment
                cudaStream_t s = A.ctx->stream;
                BT_CUDA(cudaMemcpyAsync(A.lch.p, A.bkh.p + (size_t)(len - 1) * A.vsz, A.vsz * sizeof(float2),
                                        cudaMemcpyDeviceToDevice, s));
                BT_CUDA(cudaMemcpyAsync(A.lcl.p, A.bkl.p + (size_t)(len - 1) * A.vsz, A.vsz * sizeof(float2),
                                        cudaMemcpyDeviceToDevice, s));
            }
        }
    }
}

static int adj_stride(int N, int stride) {
    if (stride <= 0) stride = (int)std::ceil(std::sqrt((double)N));
    return std::max(1, std::min(stride, N));
}

void adjoint_mixed(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq, double rtol,
                   int32_t maxit, int32_t stride, double* sig, double* dD, double* dinvT2, double* dkappa,
                   bt_stats* st, const double* weights, double* dD_cell, double* dinvT2_cell) {
    Schedule& S = ctx->sched;
    cudaStream_t s = ctx->stream;
    AdjMesh A;
    const bool cells = weights != nullptr;
    adj_mesh_setup(A, ctx, cells);
    DevBuf<double> acc6, accTc;
    if (cells) {
        acc6.alloc((size_t)ctx->mesh.n_t * 6);
        acc6.zero(s);
        accTc.alloc((size_t)ctx->mesh.n_t);
        accTc.zero(s);
        A.acc6 = acc6.p;
        A.accTc = accTc.p;
    }
    SolverMixed& W = *A.W;
    const int N = S.n_steps;
    stride = adj_stride(N, stride);
    const int nck = (N + stride - 1) / stride;
    reset_stats(st, N, rtol);
    ctx->last_iters.assign((size_t)nsig * N, 0);   // collect_batch records the forward sweep's counts
    W.saved.clear();
    W.saved_nsig = 0;
    float ms = 0.0f;
    int64_t launches = 1;
    // signals per set of launches: at most 256, and few enough that the checkpoint,
    // segment and backward states (a double-float complex value per dof each) and
    // the accumulators of a batch take at most a quarter of the free device memory
    // (the RHS padding can double the states)
    int cap = kMaxRhs / 2;
    {
        size_t free_b = 0, total_b = 0;
        BT_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const Mesh& m = ctx->mesh;
        const double per_sig = (double)((nck + 1) + (stride + 1) + stride + 1) * 16.0 * (double)m.n_dofs +
                               8.0 * (2.0 * (double)m.n_t + (double)std::max<int64_t>(1, m.n_iface));
        cap = (int)std::max(1.0, std::min((double)cap, 0.25 * (double)free_b / per_sig));
    }
    std::vector<double> kap_sig;
    if (cells && dkappa) kap_sig.assign((size_t)nsig * ctx->mesh.n_regions * ctx->mesh.n_regions, 0.0);
    BT_CUDA(cudaEventRecord(ctx->ev0, s));
    for (int32_t b0 = 0; b0 < nsig; b0 += cap) {
        const int NS = std::min<int32_t>(cap, nsig - b0);
        const int R = 2 * NS;
        if (cells) A.wsig.upload(weights + b0, NS, s);
        upload_rhs(ctx, W, NS, q + b0, gdir + 3 * b0, seq ? seq + b0 : nullptr);
        const auto geo = autotune_mixed(ctx, W, R, rtol, maxit, A.d_u0);
        adj_batch_alloc(A, NS, padded_rhs(R, geo.lpr), nck, stride);
        std::vector<AdjMesh*> G{&A};
        auto launch = [&](int n_steps, const std::vector<MixExtra>& ex) {
            return launch_batch(ctx, W, R, geo.lpr, geo.per_sm, geo.blocked, n_steps, rtol, maxit, A.d_u0, &ex[0]);
        };
        adj_pipeline(G, N, stride, S.theta, launch, {(int)b0}, {sig}, ms, launches);
        if (cells)
            adj_finish(A, b0, nullptr, nullptr, dkappa ? kap_sig.data() : nullptr);
        else
            adj_finish(A, b0, dD, dinvT2, dkappa);
    }
    if (cells) {
        const int nr2 = ctx->mesh.n_regions * ctx->mesh.n_regions;
        if (dkappa)
            for (int k = 0; k < nr2; ++k) {
                double a = 0.0;
                for (int32_t i = 0; i < nsig; ++i) a += weights[i] * kap_sig[(size_t)i * nr2 + k];
                dkappa[k] = a;
            }
        if (dD_cell) acc6.download(dD_cell, (size_t)ctx->mesh.n_t * 6, s);
        if (dinvT2_cell) accTc.download(dinvT2_cell, (size_t)ctx->mesh.n_t, s);
    }
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    BT_CUDA(cudaEventSynchronize(ctx->ev2));
    float total = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total, ctx->ev0, ctx->ev2));
    if (st) {
        st->gpu_ms = total;
        st->stepper_ms = ms;
        st->kernel_launches = launches;
    }
}

// The batched adjoint of several meshes in one call.  Meshes whose batch fills
// the GPU run alone (adjoint_mixed); the others share every launch of the
// pipeline (forward with checkpoints, the w step, segment recomputes, backward
// segments), each mesh with its own sub-grid, barriers and reductions, so small
// meshes do not each pay a whole-GPU launch per phase.
void adjoint_mixed_multi(bt_ctx* const* ctxs, int32_t nm, const int32_t* nsig, const double* q, const double* gdir,
                         const int32_t* seq, double rtol, int32_t maxit, int32_t stride, double* sig, double* dD,
                         double* dinvT2, double* dkappa, bt_stats* st) {
    bt_ctx* c0 = ctxs[0];
    cudaStream_t s = c0->stream;
    const int N = c0->sched.n_steps;
    for (int m = 0; m < nm; ++m)
        BT_REQUIRE(ctxs[m]->sched.n_steps == N && ctxs[m]->sched.theta == c0->sched.theta, BT_ERR_INVALID,
                   "bt_adjoint_multi: every mesh needs the same number of time steps and theta");
    stride = adj_stride(N, stride);
    const int nck = (N + stride - 1) / stride;
    // every mesh's work goes on the first context's stream for this call
    std::vector<cudaStream_t> saved(nm);
    for (int m = 0; m < nm; ++m) {
        BT_CUDA(cudaStreamSynchronize(ctxs[m]->stream));
        saved[m] = ctxs[m]->stream;
        ctxs[m]->stream = s;
    }
    struct Restore {
        bt_ctx* const* c;
        std::vector<cudaStream_t>& v;
        ~Restore() {
            for (size_t m = 0; m < v.size(); ++m) c[m]->stream = v[m];
        }
    } restore{ctxs, saved};
    std::vector<int64_t> off(nm + 1, 0), offr(nm + 1, 0), offk(nm + 1, 0);
    for (int m = 0; m < nm; ++m) {
        const int nr = ctxs[m]->mesh.n_regions;
        off[m + 1] = off[m] + nsig[m];
        offr[m + 1] = offr[m] + (int64_t)nsig[m] * nr;
        offk[m + 1] = offk[m] + (int64_t)nsig[m] * nr * nr;
    }
    std::vector<int> small, large;
    for (int m = 0; m < nm; ++m) {
        const int64_t units = ctxs[m]->mesh.n_dofs * (int64_t)ceil_pow2(2 * nsig[m]) / 64;
        (units / kWarpsB >= 2 * ctxs[m]->num_sms ? large : small).push_back(m);
    }
    if (small.size() == 1) {
        large.push_back(small[0]);
        small.clear();
    }
    reset_stats(st, N, rtol);
    BT_CUDA(cudaEventRecord(c0->ev3, s));
    for (int m : large) {
        bt_stats one{};
        adjoint_mixed(ctxs[m], nsig[m], q + off[m], gdir + 3 * off[m], seq ? seq + off[m] : nullptr, rtol, maxit,
                      stride, sig + off[m], dD ? dD + offr[m] : nullptr, dinvT2 ? dinvT2 + offr[m] : nullptr,
                      dkappa ? dkappa + offk[m] : nullptr, &one);
        add_stats(st, one);
    }
    if (!small.empty()) {
        const int ng = (int)small.size();
        std::vector<bt_ctx*> cs;
        std::vector<int> R;
        std::vector<const double*> u0s(ng, nullptr);
        std::vector<std::unique_ptr<AdjMesh>> As;
        for (int m : small) {
            cs.push_back(ctxs[m]);
            R.push_back(2 * nsig[m]);
            As.emplace_back(new AdjMesh());
            adj_mesh_setup(*As.back(), ctxs[m]);
            upload_rhs(ctxs[m], *As.back()->W, nsig[m], q + off[m], gdir + 3 * off[m], seq ? seq + off[m] : nullptr);
            ctxs[m]->last_iters.assign((size_t)nsig[m] * N, 0);
            As.back()->W->saved.clear();
            As.back()->W->saved_nsig = 0;
        }
        // a lanes-per-row every mesh's batch can use: the choice bt_solve_multi made
        // for this set of meshes and batch sizes, else the fastest on 3-step runs
        std::vector<int> cands;
        for (int c = 1; c <= 32; c <<= 1) {
            bool ok = true;
            for (int g = 0; g < ng; ++g) ok = ok && padded_rhs(R[g], c) > 0;
            if (ok) cands.push_back(c);
        }
        if (cs[0]->opt_mixed_lpr > 0) cands = {cs[0]->opt_mixed_lpr};
        BT_REQUIRE(!cands.empty(), BT_ERR_INVALID, "bt_adjoint_multi: no lanes-per-row fits every mesh's batch");
        int lpr = cands[0];
        std::vector<int64_t> key;
        for (int g = 0; g < ng; ++g) {
            key.push_back(cs[g]->mesh.n_dofs);
            key.push_back(R[g]);
        }
        SolverMixed& Wc = *cs[0]->smx;
        auto hit = Wc.tuned_multi.find(key);
        if (cs[0]->opt_mixed_lpr <= 0 && hit != Wc.tuned_multi.end()) {
            lpr = hit->second;
        } else if (cands.size() > 1) {
            float best = 1e30f;
            for (int c : cands) {
                const float t = launch_multi(cs.data(), ng, R, c, 3, rtol, maxit, u0s);
                if (t < best) {
                    best = t;
                    lpr = c;
                }
            }
            Wc.tuned_multi[key] = lpr;
        }
        std::vector<AdjMesh*> G;
        std::vector<int> b0(ng, 0);
        std::vector<double*> sg(ng);
        for (int g = 0; g < ng; ++g) {
            adj_batch_alloc(*As[g], nsig[small[g]], padded_rhs(R[g], lpr), nck, stride);
            G.push_back(As[g].get());
            sg[g] = sig + off[small[g]];
        }
        float ms = 0.0f;
        int64_t launches = 0;
        auto launch = [&](int n_steps, const std::vector<MixExtra>& ex) {
            return launch_multi(cs.data(), ng, R, lpr, n_steps, rtol, maxit, u0s, &ex);
        };
        adj_pipeline(G, N, stride, c0->sched.theta, launch, b0, sg, ms, launches);
        for (int g = 0; g < ng; ++g) {
            const int m = small[g];
            adj_finish(*As[g], 0, dD ? dD + offr[m] : nullptr, dinvT2 ? dinvT2 + offr[m] : nullptr,
                       dkappa ? dkappa + offk[m] : nullptr);
        }
        if (st) {
            st->stepper_ms += ms;
            st->kernel_launches += launches;
        }
    }
    BT_CUDA(cudaEventRecord(c0->ev2, s));
    BT_CUDA(cudaEventSynchronize(c0->ev2));
    float total = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total, c0->ev3, c0->ev2));
    if (st) st->gpu_ms = total;
}

}  // namespace bt
