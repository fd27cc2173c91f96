// Shared definitions of libbtgpu: error handling, device buffers, the context,
// and device helpers (complex arithmetic, warp reductions, the bounded grid
// barrier used by the persistent time-stepping kernels).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/btgpu.h"

namespace bt {

// ---------------------------------------------------------------- errors ----
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define BT_CUDA(expr)                                                              \
    do {                                                                           \
        cudaError_t e__ = (expr);                                                  \
        if (e__ != cudaSuccess) {                                                  \
            int code__ = (e__ == cudaErrorMemoryAllocation) ? BT_ERR_OOM : BT_ERR_CUDA; \
            throw ::bt::Error(code__, std::string(#expr) + ": " + cudaGetErrorString(e__) + \
                                          " (" __FILE__ ":" + std::to_string(__LINE__) + ")"); \
        }                                                                          \
    } while (0)

#define BT_REQUIRE(cond, code, msg)                                                \
    do {                                                                           \
        if (!(cond)) throw ::bt::Error((code), (msg));                             \
    } while (0)

// ----------------------------------------------------------- device buffer ----
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        BT_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    void zero(cudaStream_t s) {
        if (p) BT_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
    void upload(const T* h, size_t count, cudaStream_t s) {
        alloc(count);
        if (count) BT_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T* h, size_t count, cudaStream_t s) const {
        if (count) BT_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    operator T*() const { return p; }
};

// Device status codes written by kernels (mapped to BT_ERR_* on the host).
enum DevStatus : int {
    DEV_OK = 0,
    DEV_TIMEOUT = 1,
    DEV_NOT_CONVERGED = 2,
    DEV_BREAKDOWN = 3,
    DEV_BAD_MESH = 4,
    DEV_OVERFLOW = 5,
};

constexpr int kMaxCompartments = 8;
constexpr int kMaxColours = 256;

// ------------------------------------------------------------- the context ----
struct Solver64;     // FP64 persistent stepper workspace (stepper64.cu)
struct SolverMixed;  // batched mixed-precision workspace (batched.cu)
struct Strong;       // strong pseudo-periodic form: folded system and stepper (strong.cu)

struct Mesh {
    int64_t n_v = 0, n_t = 0;
    int32_t n_regions = 0, n_comp = 0;
    std::vector<int32_t> region_comp;  // host copy
    DevBuf<double> xyz;
    DevBuf<int32_t> tets, region, comp;
    // duplicated-node graph
    int64_t n_dofs = 0, nnz = 0, n_iface = 0;
    DevBuf<int32_t> dof_of;        // [n_v * n_comp], -1 when dead
    DevBuf<int32_t> dof_vertex, dof_comp;
    DevBuf<int32_t> vt_ptr, vt_list;  // vertex -> cells (sorted)
    DevBuf<int32_t> nbr;              // [n_t*4] cell across face a (opposite local vertex a), -1 boundary
    DevBuf<int32_t> row_ptr, col;     // CSR
    DevBuf<int32_t> diag_pos;         // CSR position of the diagonal of each row
    DevBuf<int32_t> iface_cell, iface_face;  // interface facets: owning (lower-index) cell, local face
    // cell colouring
    int32_t n_colours = 0;
    std::vector<int32_t> colour_ptr;  // host, n_colours+1
    DevBuf<int32_t> colour, colour_cells;
    // sliced ELL (C = 32)
    int32_t n_slices = 0;
    int64_t sell_entries = 0;
    DevBuf<int32_t> sl_ptr, sl_w, sl_col, sl_pos;  // sl_pos: CSR position or -1 (padding)
    double volume = 0.0;
    bool built = false;
};

struct Coeffs {
    DevBuf<double> D_region, invT2_region, kappa_pair, D_cell, invT2_cell;
    bool has_cell_D = false;
    bool has_cell_T2 = false;
    bool kappa_cr = false;   // Crouzeix-Raviart (per-facet linear) permeability
    bool set = false;
};

struct Assembled {
    DevBuf<double> M, K, T, R, Jx, Jy, Jz;  // CSR order
    DevBuf<double> w;                       // signal weight per dof
    DevBuf<double> vw;                      // int phi_v over the whole mesh, per vertex
    bool done = false;
    int64_t version = 0;                    // incremented by every assembly
};

struct Schedule {
    std::vector<double> f_new, f_old;  // [n_seq * n_steps]
    std::vector<double> F_old;         // integral F = int_0^t f at the explicit level (pseudo-periodic phase)
    std::vector<double> F_new;         // F at the implicit level (strong pseudo-periodic form)
    int32_t n_steps = 0, n_seq = 0;
    double dt = 0.0, theta = 0.5;
    bool set = false;
    bool phase_set = false;
};

// One mirror-term entry of a boundary row: coefficient and the shift of the
// boundary vertex to its mirror point.
struct alignas(16) PerVal {
    double c, x, y, z;
};

// Weak pseudo-periodic boundaries (penalty form, periodic.cu): the implicit
// matrix gains theta * PB, PB_ij = int_{exterior facets} kappa_e phi_i phi_j with
// kappa_e the P1 interpolant of 3e-3/hmin on the periodic faces; every step's
// right-hand side gains (1 - theta) sum_e val.c e^{i q F(tp) g.(val.x,val.y,val.z)} u_n[col]
// over the entries of the row (PB_ij times the weight of mirror dof k in the
// mirror point of vertex j, and the shift of vertex j).
struct Periodic {
    bool on = false;
    int32_t dir[3] = {0, 0, 0};
    double kappa_e = 0.0, hmin = 0.0;
    int64_t n_facets = 0, n_rows = 0, n_entries = 0, n_unmatched = 0;
    DevBuf<double> PB;            // CSR order
    DevBuf<int32_t> ptr, col;     // [n_dofs + 1], [n_entries]
    DevBuf<PerVal> val;           // [n_entries]
};

}  // namespace bt

struct bt_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    int num_sms = 0;
    bt::Mesh mesh;
    bt::Coeffs coeffs;
    bt::Assembled mat;
    bt::Schedule sched;
    bt::Periodic per;
    bt::Solver64* s64 = nullptr;
    bt::SolverMixed* smx = nullptr;
    bt::Strong* strong = nullptr;
    int periodic_mode = 0;            // BT_PERIODIC_WEAK or BT_PERIODIC_STRONG
    bool last_strong = false;         // the last solve ran the strong pseudo-periodic stepper
    // last solve
    int32_t last_nsig = 0;
    int32_t last_precision = -1;
    std::vector<int32_t> last_iters;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    // tuning knobs (bt_set_option); negative = automatic
    int opt_mixed_lpr = -1;
    int opt_mixed_blocks_per_sm = -1;
    int opt_mixed_max_sweeps = 8;
    double opt_mixed_eps_first = 3e-6;
    double opt_mixed_eps_next = 1e-2;
    int opt_mixed_extrapolate = 4;   // order of the mixed path's extrapolated initial guess (0..4)
    int opt_mixed_blocked = -1;
    int opt_mixed_reduce = -1;
    double opt_mixed_growth2 = 1e8;   // divergence guard of a sweep (squared-norm growth over its minimum)
    int opt_fp64_extrapolate = 4;    // order of the FP64 path's extrapolated initial guess (0..4)
    int opt_fp64_pair = 2;            // FP64 path: two signals of one direction share a launch (0: off)
    int opt_fp64_blocks_per_sm = -1;  // FP64 one-signal stepper: blocks per SM cap (0: as many as fit, -1: auto)
    int opt_mixed_inner = 2;          // grid-wide reductions per inner COCG iteration: 1 or 2
    int opt_mixed_sort = 1;           // order a solve's signals by (sequence, |q|) before batching
    int opt_strong_batch = 1;         // strong form: signals of one direction share a batched launch
    // failure detection: time limit of every device-side wait, and a switch that
    // makes the next solve's first wait run out (see stalled_wait)
    unsigned long long opt_wait_ns = 2000000000ull;
    int opt_stall_first_wait = 0;
};

namespace bt {

// Host entry points of the translation units.
void build_graph(bt_ctx* ctx, const double* xyz, int64_t n_v, const int32_t* tets, int64_t n_t,
                 const int32_t* region, int32_t n_regions, const int32_t* region_comp);
void assemble_all(bt_ctx* ctx);
void solve_fp64(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq,
                const double* u0, double rtol, int32_t maxit, double* sig, double* comp_sig,
                bt_stats* st);
void solve_mixed(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq,
                 const double* u0, double rtol, int32_t maxit, double* sig, double* comp_sig,
                 bt_stats* st);
void get_solution_fp64(bt_ctx* ctx, int32_t index, double* u);
void adjoint_fp64(bt_ctx* ctx, double q, const double* gdir, int32_t seq, const double* u0, double rtol,
                  int32_t maxit, int32_t stride, double* sig, double* dD, double* dinvT2, double* dkappa,
                  bt_stats* st,
                  double* dD_cell = nullptr, double* dinvT2_cell = nullptr);
void get_solution_mixed(bt_ctx* ctx, int32_t index, double* u);
void tangent_fp64(bt_ctx* ctx, double q, const double* gdir, int32_t seq, const double* u0, int32_t kind, int32_t ri,
                  int32_t rj, double rtol, int32_t maxit, double* sig, double* dsig, bt_stats* st);
void solve_mixed_multi(bt_ctx* const* ctxs, int32_t n_meshes, const int32_t* nsig, const double* q,
                       const double* gdir, const int32_t* seq, double rtol, int32_t maxit, double* sig,
                       bt_stats* st);
void reset_tuning_mixed(bt_ctx* ctx);
void set_periodic(bt_ctx* ctx, const int32_t* dir);
void set_strong(bt_ctx* ctx, const int32_t* dir);
bool strong_active(const bt_ctx* ctx);
void solve_strong(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq,
                  const double* u0, double rtol, int32_t maxit, double* sig, double* comp_sig, bt_stats* st);
void get_solution_strong(bt_ctx* ctx, int32_t index, double* u);
void strong_info(const bt_ctx* ctx, int64_t* n_dofs, int64_t* nnz, int64_t* n_classes);
void free_strong(bt_ctx* ctx);
void strong_directions(const bt_ctx* ctx, int32_t* dir);
void adjoint_mixed(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq, double rtol,
                   int32_t maxit, int32_t stride, double* sig, double* dD, double* dinvT2, double* dkappa,
                   bt_stats* st,
                   const double* weights = nullptr, double* dD_cell = nullptr, double* dinvT2_cell = nullptr);
void adjoint_mixed_multi(bt_ctx* const* ctxs, int32_t nm, const int32_t* nsig, const double* q, const double* gdir,
                         const int32_t* seq, double rtol, int32_t maxit, int32_t stride, double* sig, double* dD,
                         double* dinvT2, double* dkappa, bt_stats* st);

void free_solvers(bt_ctx* ctx);
double device_sum(const double* d, int64_t n, cudaStream_t s);
double device_dot(const double* a, const double* b, int64_t n, cudaStream_t s);
void exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int32_t* total_out,
                        cudaStream_t s);

// ------------------------------------------------------------ device helpers --
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 cinv(double2 b) {
    double d = b.x * b.x + b.y * b.y;
    return make_double2(b.x / d, -b.y / d);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acqrel_u32(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long atom_add_acqrel_u64(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.add.acq_rel.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier for cooperative (co-resident) launches.  bar[0] counts
// arrivals, bar[1] is the generation.  Every wait is bounded: after
// kBarrierTimeoutNs (or kBarrierMaxSpins polls) the block records DEV_TIMEOUT
// in *status and the function returns false so the caller can leave the
// kernel; a block that finds *status already set leaves at once.
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s
constexpr unsigned kBarrierMaxSpins = 1u << 26;

__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* status,
                                             unsigned& gen, unsigned long long limit_ns = kBarrierTimeoutNs) {
    __shared__ int s_ok;
    __threadfence();   // each thread's own stores are device-visible before its block arrives
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned target = gen + 1;
        __threadfence();
        if (ld_relaxed_i32(status) != DEV_OK) {
            ok = 0;
        } else {
            unsigned arrived = atom_add_acqrel_u32(&bar[0], 1u);
            if (arrived == nblocks - 1) {
                bar[0] = 0;
                st_release_u32(&bar[1], target);
            } else {
                const unsigned long long t0 = globaltimer_ns();
                unsigned spins = 0;
                while (ld_acquire_u32(&bar[1]) != target) {
                    if (++spins > kBarrierMaxSpins || (spins & 255u) == 0u &&
                        (globaltimer_ns() - t0 > limit_ns || ld_relaxed_i32(status) != DEV_OK)) {
                        atomicCAS(status, DEV_OK, DEV_TIMEOUT);
                        ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
            }
        }
        __threadfence();
        gen = target;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Failure-detection hook (option "test.stall_first_wait"): thread 0 of every
// block waits for a word that nothing in the launch writes (never[0], zeroed
// before the launch), so the wait runs out after limit_ns (or the poll limit),
// records DEV_TIMEOUT in *status and every block leaves the kernel; the host
// then reports BT_ERR_TIMEOUT and the context stays usable.  Returns false.
__device__ __forceinline__ bool stalled_wait(const unsigned* never, int* status, unsigned long long limit_ns) {
    if (threadIdx.x == 0) {
        const unsigned long long t0 = globaltimer_ns();
        unsigned spins = 0;
        while (ld_acquire_u32(never) != 1u) {
            if (++spins > kBarrierMaxSpins || (spins & 255u) == 0u &&
                (globaltimer_ns() - t0 > limit_ns || ld_relaxed_i32(status) != DEV_OK)) {
                atomicCAS(status, DEV_OK, DEV_TIMEOUT);
                break;
            }
            __nanosleep(32);
        }
    }
    __syncthreads();
    return false;
}

// Block-wide sum of NV doubles; the deterministic result is v[] of thread 0
// (blockDim a multiple of 32).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* [32*NV] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) smem[wid * NV + k] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = (lane < nw) ? smem[lane * NV + k] : 0.0;
            v[k] = warp_sum(t);
        }
    }
    __syncthreads();
}

// All blocks: deterministic sum over nblocks partials (fixed order), result in
// smem_out[k] for every thread of the block.
template <int NV>
__device__ __forceinline__ void grid_partials_sum(const double* partials, int nblocks, double* smem_out) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (wid == 0) {
        double acc[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = 0.0;
        for (int b = lane; b < nblocks; b += 32) {
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&partials[(size_t)b * NV + k]);
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = warp_sum(acc[k]);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) smem_out[k] = acc[k];
        }
    }
    __syncthreads();
}

}  // namespace bt
