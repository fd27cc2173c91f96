// extern "C" entry points of libbtgpu (declared in include/btgpu.h).  Every
// function converts exceptions into a status code and records the message in
// the context; nothing here calls exit().
#include "bt_common.cuh"

#include <nvtx3/nvToolsExt.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace bt {
void free_solver64(bt_ctx* ctx);
void free_solver_mixed(bt_ctx* ctx);
}  // namespace bt

namespace {

// NVTX range around an entry point (visible in Nsight Systems / ncu range filters;
// a no-op without an attached tool).
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

template <typename F>
int guarded(bt_ctx* ctx, F&& f) {
    try {
        f();
        if (ctx) ctx->err.clear();
        return BT_OK;
    } catch (const bt::Error& e) {
        if (ctx) ctx->err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->err = "host allocation failed";
        return BT_ERR_OOM;
    } catch (const std::exception& e) {
        if (ctx) ctx->err = e.what();
        return BT_ERR_INVALID;
    }
}

void use_device(bt_ctx* ctx) { BT_CUDA(cudaSetDevice(ctx->device)); }

}  // namespace



extern "C" {

int bt_version(void) { return 100; }

int bt_create(bt_ctx** out, int device) {
    if (!out) return BT_ERR_INVALID;
    *out = nullptr;
    bt_ctx* ctx = nullptr;
    try {
        ctx = new bt_ctx();
    } catch (...) {
        return BT_ERR_OOM;
    }
    ctx->device = device;
    int rc = guarded(ctx, [&] {
        int ndev = 0;
        BT_CUDA(cudaGetDeviceCount(&ndev));
        BT_REQUIRE(device >= 0 && device < ndev, BT_ERR_INVALID, "no such CUDA device");
        use_device(ctx);
        BT_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
        ctx->stream = ctx->own_stream;
        BT_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
        int coop = 0;
        BT_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
        BT_REQUIRE(coop, BT_ERR_CUDA, "device does not support cooperative launches");
        BT_CUDA(cudaEventCreate(&ctx->ev0));
        BT_CUDA(cudaEventCreate(&ctx->ev1));
        BT_CUDA(cudaEventCreate(&ctx->ev2));
        BT_CUDA(cudaEventCreate(&ctx->ev3));
    });
    if (rc != BT_OK) {
        bt_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return BT_OK;
}

int bt_destroy(bt_ctx* ctx) {
    if (!ctx) return BT_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    bt::free_solver64(ctx);
    bt::free_solver_mixed(ctx);
    bt::free_strong(ctx);
    ctx->mesh = bt::Mesh();
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev2) cudaEventDestroy(ctx->ev2);
    if (ctx->ev3) cudaEventDestroy(ctx->ev3);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return BT_OK;
}

int bt_last_error(const bt_ctx* ctx, char* buf, size_t len) {
    if (!ctx || !buf || len == 0) return BT_ERR_INVALID;
    std::strncpy(buf, ctx->err.c_str(), len - 1);
    buf[len - 1] = '\0';
    return BT_OK;
}

int bt_set_stream(bt_ctx* ctx, void* cuda_stream) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        use_device(ctx);
        BT_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->stream = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
    });
}

int bt_mesh_upload(bt_ctx* ctx, const double* xyz, int64_t n_vertices, const int32_t* tets, int64_t n_cells,
                   const int32_t* cell_region, int32_t n_regions, const int32_t* region_compartment) {
    Range range_("bt_mesh_upload");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(xyz && tets && cell_region, BT_ERR_INVALID, "bt_mesh_upload: NULL array");
        use_device(ctx);
        ctx->mat.done = false;
        ctx->coeffs = bt::Coeffs();
        ctx->per = bt::Periodic();
        ctx->periodic_mode = BT_PERIODIC_WEAK;
        bt::free_strong(ctx);
        bt::free_solver64(ctx);
        bt::free_solver_mixed(ctx);
        bt::build_graph(ctx, xyz, n_vertices, tets, n_cells, cell_region, n_regions, region_compartment);
    });
}

int bt_mesh_info(bt_ctx* ctx, bt_mesh_info_t* out) {
    if (!ctx || !out) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Mesh& m = ctx->mesh;
        BT_REQUIRE(m.built, BT_ERR_STATE, "bt_mesh_info: no mesh");
        out->n_vertices = m.n_v;
        out->n_cells = m.n_t;
        out->n_dofs = m.n_dofs;
        out->nnz = m.nnz;
        out->n_interface_facets = m.n_iface;
        out->n_compartments = m.n_comp;
        out->n_colours = m.n_colours;
        out->sell_entries = m.sell_entries;
        out->volume = m.volume;
    });
}

int bt_set_coefficients(bt_ctx* ctx, const double* D_region, const double* invT2_region,
                        const double* kappa_pair) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Mesh& m = ctx->mesh;
        BT_REQUIRE(m.built, BT_ERR_STATE, "bt_set_coefficients: no mesh");
        BT_REQUIRE(D_region, BT_ERR_INVALID, "bt_set_coefficients: D_region is NULL");
        use_device(ctx);
        const int nr = m.n_regions;
        std::vector<double> D(D_region, D_region + nr), iT2(nr, 0.0), kp((size_t)nr * nr, 0.0);
        for (int r = 0; r < nr; ++r) BT_REQUIRE(std::isfinite(D[r]) && D[r] >= 0.0, BT_ERR_INVALID, "D must be finite and >= 0");
        if (invT2_region)
            for (int r = 0; r < nr; ++r) {
                iT2[r] = invT2_region[r];
                BT_REQUIRE(std::isfinite(iT2[r]) && iT2[r] >= 0.0, BT_ERR_INVALID, "1/T2 must be finite and >= 0");
            }
        if (kappa_pair)
            for (int i = 0; i < nr * nr; ++i) {
                kp[i] = kappa_pair[i];
                BT_REQUIRE(std::isfinite(kp[i]) && kp[i] >= 0.0, BT_ERR_INVALID, "kappa must be finite and >= 0");
            }
        for (int i = 0; i < nr; ++i)
            for (int j = 0; j < nr; ++j)
                BT_REQUIRE(kp[(size_t)i * nr + j] == kp[(size_t)j * nr + i], BT_ERR_INVALID, "kappa_pair must be symmetric");
        bt::Coeffs& c = ctx->coeffs;
        c.D_region.upload(D.data(), nr, ctx->stream);
        c.invT2_region.upload(iT2.data(), nr, ctx->stream);
        c.kappa_pair.upload(kp.data(), (size_t)nr * nr, ctx->stream);
        BT_CUDA(cudaStreamSynchronize(ctx->stream));
        c.set = true;
        ctx->mat.done = false;
    });
}

int bt_set_kappa_mode(bt_ctx* ctx, int32_t mode) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built, BT_ERR_STATE, "bt_set_kappa_mode: no mesh");
        BT_REQUIRE(mode == BT_KAPPA_FACET || mode == BT_KAPPA_CR, BT_ERR_INVALID,
                   "bt_set_kappa_mode: mode must be BT_KAPPA_FACET or BT_KAPPA_CR");
        ctx->coeffs.kappa_cr = (mode == BT_KAPPA_CR);
        ctx->mat.done = false;
    });
}

int bt_set_cell_diffusion(bt_ctx* ctx, const double* D_cell) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Mesh& m = ctx->mesh;
        BT_REQUIRE(m.built, BT_ERR_STATE, "bt_set_cell_diffusion: no mesh");
        use_device(ctx);
        bt::Coeffs& c = ctx->coeffs;
        if (!D_cell) {
            c.D_cell.release();
            c.has_cell_D = false;
        } else {
            for (int64_t i = 0; i < m.n_t * 6; ++i)
                BT_REQUIRE(std::isfinite(D_cell[i]), BT_ERR_INVALID, "D_cell must be finite");
            c.D_cell.upload(D_cell, (size_t)m.n_t * 6, ctx->stream);
            BT_CUDA(cudaStreamSynchronize(ctx->stream));
            c.has_cell_D = true;
        }
        ctx->mat.done = false;
    });
}

int bt_set_cell_T2(bt_ctx* ctx, const double* invT2_cell) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Mesh& m = ctx->mesh;
        BT_REQUIRE(m.built, BT_ERR_STATE, "bt_set_cell_T2: no mesh");
        use_device(ctx);
        bt::Coeffs& c = ctx->coeffs;
        if (!invT2_cell) {
            c.invT2_cell.release();
            c.has_cell_T2 = false;
        } else {
            for (int64_t i = 0; i < m.n_t; ++i)
                BT_REQUIRE(std::isfinite(invT2_cell[i]) && invT2_cell[i] >= 0.0, BT_ERR_INVALID,
                           "invT2_cell must be finite and >= 0");
            c.invT2_cell.upload(invT2_cell, (size_t)m.n_t, ctx->stream);
            BT_CUDA(cudaStreamSynchronize(ctx->stream));
            c.has_cell_T2 = true;
        }
        ctx->mat.done = false;
    });
}

int bt_assemble(bt_ctx* ctx) {
    Range range_("bt_assemble");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        use_device(ctx);
        bt::assemble_all(ctx);
    });
}

int bt_set_schedule(bt_ctx* ctx, const double* f_new, const double* f_old, int32_t n_steps, int32_t n_sequences,
                    double dt, double theta) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(f_new && f_old, BT_ERR_INVALID, "bt_set_schedule: NULL schedule");
        BT_REQUIRE(n_steps >= 1 && n_sequences >= 1, BT_ERR_INVALID, "bt_set_schedule: empty schedule");
        BT_REQUIRE(std::isfinite(dt) && dt > 0.0, BT_ERR_INVALID, "dt must be > 0");
        BT_REQUIRE(std::isfinite(theta) && theta > 0.0 && theta <= 1.0, BT_ERR_INVALID, "theta must be in (0, 1]");
        const size_t n = (size_t)n_steps * n_sequences;
        for (size_t i = 0; i < n; ++i)
            BT_REQUIRE(std::isfinite(f_new[i]) && std::isfinite(f_old[i]), BT_ERR_INVALID, "schedule must be finite");
        bt::Schedule& S = ctx->sched;
        S.f_new.assign(f_new, f_new + n);
        S.f_old.assign(f_old, f_old + n);
        S.n_steps = n_steps;
        S.n_seq = n_sequences;
        S.dt = dt;
        S.theta = theta;
        S.set = true;
        S.F_old.clear();
        S.F_new.clear();
        S.phase_set = false;
    });
}

int bt_set_schedule_phase(bt_ctx* ctx, const double* F_old, int32_t n_steps, int32_t n_sequences) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        bt::Schedule& S = ctx->sched;
        BT_REQUIRE(S.set, BT_ERR_STATE, "bt_set_schedule_phase: call bt_set_schedule first");
        BT_REQUIRE(F_old, BT_ERR_INVALID, "bt_set_schedule_phase: NULL array");
        BT_REQUIRE(n_steps == S.n_steps && n_sequences == S.n_seq, BT_ERR_INVALID,
                   "bt_set_schedule_phase: sizes differ from the schedule");
        const size_t n = (size_t)n_steps * n_sequences;
        for (size_t i = 0; i < n; ++i)
            BT_REQUIRE(std::isfinite(F_old[i]), BT_ERR_INVALID, "bt_set_schedule_phase: values must be finite");
        S.F_old.assign(F_old, F_old + n);
        S.phase_set = true;
    });
}

int bt_set_schedule_integral(bt_ctx* ctx, const double* F_new, const double* F_old, int32_t n_steps,
                             int32_t n_sequences) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        bt::Schedule& S = ctx->sched;
        BT_REQUIRE(S.set, BT_ERR_STATE, "bt_set_schedule_integral: call bt_set_schedule first");
        BT_REQUIRE(F_new && F_old, BT_ERR_INVALID, "bt_set_schedule_integral: NULL array");
        BT_REQUIRE(n_steps == S.n_steps && n_sequences == S.n_seq, BT_ERR_INVALID,
                   "bt_set_schedule_integral: sizes differ from the schedule");
        const size_t n = (size_t)n_steps * n_sequences;
        for (size_t i = 0; i < n; ++i)
            BT_REQUIRE(std::isfinite(F_new[i]) && std::isfinite(F_old[i]), BT_ERR_INVALID,
                       "bt_set_schedule_integral: values must be finite");
        S.F_new.assign(F_new, F_new + n);
        S.F_old.assign(F_old, F_old + n);
        S.phase_set = true;
    });
}

// The directions last given to bt_set_periodic (weak or strong form).
static void apply_periodic(bt_ctx* ctx, const int32_t* dir) {
    const int32_t off[3] = {0, 0, 0};
    bt::free_solver_mixed(ctx);   // cached tuning and packed matrices do not hold the boundary term
    if (ctx->periodic_mode == BT_PERIODIC_STRONG) {
        bt::set_periodic(ctx, off);
        bt::set_strong(ctx, dir);
    } else {
        bt::free_strong(ctx);
        bt::set_periodic(ctx, dir);
    }
}

int bt_set_periodic(bt_ctx* ctx, const int32_t* periodic_dir) {
    Range range_("bt_set_periodic");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built, BT_ERR_STATE, "bt_set_periodic: no mesh");
        const int32_t off[3] = {0, 0, 0};
        use_device(ctx);
        apply_periodic(ctx, periodic_dir ? periodic_dir : off);
    });
}

int bt_set_periodic_mode(bt_ctx* ctx, int32_t mode) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(mode == BT_PERIODIC_WEAK || mode == BT_PERIODIC_STRONG, BT_ERR_INVALID,
                   "bt_set_periodic_mode: mode must be BT_PERIODIC_WEAK or BT_PERIODIC_STRONG");
        BT_REQUIRE(ctx->mesh.built, BT_ERR_STATE, "bt_set_periodic_mode: no mesh");
        use_device(ctx);
        int32_t dir[3] = {0, 0, 0};
        for (int d = 0; d < 3; ++d)
            dir[d] = ctx->per.dir[d];
        if (ctx->periodic_mode == BT_PERIODIC_STRONG) bt::strong_directions(ctx, dir);
        ctx->periodic_mode = mode;
        apply_periodic(ctx, dir);
    });
}

int bt_strong_periodic_info(bt_ctx* ctx, int64_t* n_dofs, int64_t* nnz, int64_t* n_classes) {
    if (!ctx || !n_dofs || !nnz || !n_classes) return BT_ERR_INVALID;
    return guarded(ctx, [&] { bt::strong_info(ctx, n_dofs, nnz, n_classes); });
}

int bt_periodic_info(bt_ctx* ctx, bt_periodic_info_t* out) {
    if (!ctx || !out) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Periodic& P = ctx->per;
        out->active = P.on ? 1 : 0;
        for (int d = 0; d < 3; ++d) out->dir[d] = P.dir[d];
        out->kappa_e = P.kappa_e;
        out->hmin = P.hmin;
        out->n_facets = P.n_facets;
        out->n_rows = P.n_rows;
        out->n_entries = P.n_entries;
        out->n_unmatched = P.n_unmatched;
    });
}

int bt_solve(bt_ctx* ctx, int32_t n_signals, const double* q, const double* gdir, const int32_t* sequence,
             const double* u0, int32_t precision, double rtol, int32_t max_iterations, double* signal_out,
             double* compartment_out, double* S0_out, bt_stats* stats) {
    Range range_("bt_solve");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built && ctx->mat.done, BT_ERR_STATE, "bt_solve: mesh not assembled");
        BT_REQUIRE(ctx->sched.set, BT_ERR_STATE, "bt_solve: no schedule");
        BT_REQUIRE(n_signals >= 1 && q && gdir && signal_out, BT_ERR_INVALID, "bt_solve: bad arguments");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_solve: rtol must be > 0 and max_iterations >= 1");
        for (int32_t i = 0; i < n_signals; ++i) {
            BT_REQUIRE(std::isfinite(q[i]), BT_ERR_INVALID, "bt_solve: q must be finite");
            const double g0 = gdir[3 * i], g1 = gdir[3 * i + 1], g2 = gdir[3 * i + 2];
            BT_REQUIRE(std::isfinite(g0) && std::isfinite(g1) && std::isfinite(g2), BT_ERR_INVALID,
                       "bt_solve: gradient direction must be finite");
        }
        if (u0)
            for (int64_t v = 0; v < ctx->mesh.n_v; ++v)
                BT_REQUIRE(std::isfinite(u0[v]), BT_ERR_INVALID, "bt_solve: u0 must be finite");
        use_device(ctx);
        ctx->last_precision = -1;
        ctx->last_strong = false;
        if (bt::strong_active(ctx)) {
            BT_REQUIRE(precision == BT_PRECISION_FP64, BT_ERR_INVALID,
                       "bt_solve: the strong pseudo-periodic form runs on the FP64 path only");
            bt::solve_strong(ctx, n_signals, q, gdir, sequence, u0, rtol, max_iterations, signal_out,
                             compartment_out, stats);
            ctx->last_strong = true;
        } else if (precision == BT_PRECISION_FP64) {
            bt::solve_fp64(ctx, n_signals, q, gdir, sequence, u0, rtol, max_iterations, signal_out,
                           compartment_out, stats);
        } else if (precision == BT_PRECISION_MIXED) {
            bt::solve_mixed(ctx, n_signals, q, gdir, sequence, u0, rtol, max_iterations, signal_out,
                            compartment_out, stats);
        } else {
            throw bt::Error(BT_ERR_INVALID, "bt_solve: unknown precision");
        }
        ctx->last_precision = precision;
        if (S0_out) {
            if (u0) {
                bt::DevBuf<double> d;
                d.upload(u0, ctx->mesh.n_v, ctx->stream);
                *S0_out = bt::device_dot(ctx->mat.vw, d, ctx->mesh.n_v, ctx->stream);
            } else {
                *S0_out = ctx->mesh.volume;
            }
        }
    });
}

// Device-pointer variant of bt_solve: the per-signal parameters and u0 are read
// from device memory (staged through the host, where the solve validates them and
// builds its schedule), the signals are written to device memory on the
// context's stream.
static bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int bt_solve_dev(bt_ctx* ctx, int32_t n_signals, const double* d_q, const double* d_gdir, const int32_t* d_sequence,
                 const double* d_u0, int32_t precision, double rtol, int32_t max_iterations, double* d_signal_out,
                 double* d_compartment_out, double* S0_out, bt_stats* stats) {
    Range range_("bt_solve_dev");
    if (!ctx) return BT_ERR_INVALID;
    std::vector<double> q, g, u0, sig, comp;
    std::vector<int32_t> seq;
    int rc = guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built, BT_ERR_STATE, "bt_solve_dev: no mesh");
        BT_REQUIRE(n_signals >= 1 && d_q && d_gdir && d_signal_out, BT_ERR_INVALID, "bt_solve_dev: bad arguments");
        use_device(ctx);
        for (const void* p : {(const void*)d_q, (const void*)d_gdir, (const void*)d_signal_out})
            BT_REQUIRE(is_device_ptr(p), BT_ERR_INVALID, "bt_solve_dev: q, gdir and signal_out must be device pointers");
        BT_REQUIRE(!d_sequence || is_device_ptr(d_sequence), BT_ERR_INVALID, "bt_solve_dev: sequence must be a device pointer");
        BT_REQUIRE(!d_u0 || is_device_ptr(d_u0), BT_ERR_INVALID, "bt_solve_dev: u0 must be a device pointer");
        BT_REQUIRE(!d_compartment_out || is_device_ptr(d_compartment_out), BT_ERR_INVALID,
                   "bt_solve_dev: compartment_out must be a device pointer");
        cudaStream_t s = ctx->stream;
        q.resize(n_signals);
        g.resize((size_t)3 * n_signals);
        BT_CUDA(cudaMemcpyAsync(q.data(), d_q, q.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        BT_CUDA(cudaMemcpyAsync(g.data(), d_gdir, g.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (d_sequence) {
            seq.resize(n_signals);
            BT_CUDA(cudaMemcpyAsync(seq.data(), d_sequence, seq.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        }
        if (d_u0) {
            u0.resize(ctx->mesh.n_v);
            BT_CUDA(cudaMemcpyAsync(u0.data(), d_u0, u0.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        BT_CUDA(cudaStreamSynchronize(s));
        sig.resize(n_signals);
        comp.resize((size_t)n_signals * ctx->mesh.n_comp);
    });
    if (rc != BT_OK) return rc;
    rc = bt_solve(ctx, n_signals, q.data(), g.data(), d_sequence ? seq.data() : nullptr, d_u0 ? u0.data() : nullptr,
                  precision, rtol, max_iterations, sig.data(), d_compartment_out ? comp.data() : nullptr, S0_out,
                  stats);
    if (rc != BT_OK) return rc;
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        BT_CUDA(cudaMemcpyAsync(d_signal_out, sig.data(), sig.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        if (d_compartment_out)
            BT_CUDA(cudaMemcpyAsync(d_compartment_out, comp.data(), comp.size() * sizeof(double),
                                    cudaMemcpyHostToDevice, s));
        BT_CUDA(cudaStreamSynchronize(s));   // the host staging buffers go out of scope
    });
}

int bt_solve_multi(bt_ctx* const* contexts, int32_t n_meshes, const int32_t* n_signals, const double* q,
                   const double* gdir, const int32_t* sequence, double rtol, int32_t max_iterations,
                   double* signal_out, double* S0_out, bt_stats* stats) {
    Range range_("bt_solve_multi");
    if (!contexts || n_meshes < 1 || !contexts[0]) return BT_ERR_INVALID;
    bt_ctx* c0 = contexts[0];
    return guarded(c0, [&] {
        BT_REQUIRE(n_meshes <= 64 && n_signals && q && gdir && signal_out, BT_ERR_INVALID,
                   "bt_solve_multi: bad arguments (at most 64 meshes)");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_solve_multi: rtol must be > 0 and max_iterations >= 1");
        int64_t total = 0;
        for (int32_t m = 0; m < n_meshes; ++m) {
            bt_ctx* c = contexts[m];
            BT_REQUIRE(c != nullptr, BT_ERR_INVALID, "bt_solve_multi: null context");
            for (int32_t j = 0; j < m; ++j)
                BT_REQUIRE(contexts[j] != c, BT_ERR_INVALID, "bt_solve_multi: a context is listed twice");
            BT_REQUIRE(c->device == c0->device, BT_ERR_INVALID, "bt_solve_multi: contexts on different devices");
            BT_REQUIRE(c->mesh.built && c->mat.done && c->sched.set, BT_ERR_STATE,
                       "bt_solve_multi: every mesh needs bt_assemble and bt_set_schedule");
            BT_REQUIRE(n_signals[m] >= 1 && n_signals[m] <= 256, BT_ERR_INVALID,
                       "bt_solve_multi: 1..256 signals per mesh");
            BT_REQUIRE(!bt::strong_active(c), BT_ERR_STATE,
                       "bt_solve_multi: the strong pseudo-periodic form runs on the FP64 path (bt_solve) only");
            total += n_signals[m];
        }
        for (int64_t i = 0; i < total; ++i) {
            BT_REQUIRE(std::isfinite(q[i]) && std::isfinite(gdir[3 * i]) && std::isfinite(gdir[3 * i + 1]) &&
                           std::isfinite(gdir[3 * i + 2]),
                       BT_ERR_INVALID, "bt_solve_multi: q and gradient directions must be finite");
            if (sequence) {
                int64_t acc = 0;
                int32_t m = 0;
                while (acc + n_signals[m] <= i) acc += n_signals[m++];
                BT_REQUIRE(sequence[i] >= 0 && sequence[i] < contexts[m]->sched.n_seq, BT_ERR_INVALID,
                           "bt_solve_multi: sequence index out of range");
            }
        }
        use_device(c0);
        for (int32_t m = 0; m < n_meshes; ++m) contexts[m]->last_precision = -1;
        bt::solve_mixed_multi(contexts, n_meshes, n_signals, q, gdir, sequence, rtol, max_iterations, signal_out,
                              stats);
        for (int32_t m = 0; m < n_meshes; ++m) {
            contexts[m]->last_precision = BT_PRECISION_MIXED;
            if (S0_out) S0_out[m] = contexts[m]->mesh.volume;
        }
    });
}

int bt_tangent(bt_ctx* ctx, double q, const double* gdir, int32_t sequence, const double* u0, int32_t param,
               int32_t i, int32_t j, double rtol, int32_t max_iterations, double* signal_out, double* dsignal_out,
               bt_stats* stats) {
    Range range_("bt_tangent");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built && ctx->mat.done, BT_ERR_STATE, "bt_tangent: mesh not assembled");
        BT_REQUIRE(!bt::strong_active(ctx), BT_ERR_STATE, "bt_tangent: not defined with the strong pseudo-periodic form");
        BT_REQUIRE(ctx->sched.set, BT_ERR_STATE, "bt_tangent: no schedule");
        BT_REQUIRE(gdir && signal_out && dsignal_out, BT_ERR_INVALID, "bt_tangent: bad arguments");
        BT_REQUIRE(std::isfinite(q) && std::isfinite(gdir[0]) && std::isfinite(gdir[1]) && std::isfinite(gdir[2]),
                   BT_ERR_INVALID, "bt_tangent: q and gdir must be finite");
        BT_REQUIRE(sequence >= 0 && sequence < ctx->sched.n_seq, BT_ERR_INVALID, "bt_tangent: bad sequence");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_tangent: rtol must be > 0 and max_iterations >= 1");
        use_device(ctx);
        ctx->last_precision = -1;
        bt::tangent_fp64(ctx, q, gdir, sequence, u0, param, i, j, rtol, max_iterations, signal_out, dsignal_out,
                         stats);   // the stepper now holds the tangent state: no solution to report
    });
}

int bt_adjoint(bt_ctx* ctx, double q, const double* gdir, int32_t sequence, const double* u0, double rtol,
               int32_t max_iterations, int32_t checkpoint_stride, double* signal_out, double* dS_dD,
               double* dS_dinvT2, double* dS_dkappa, bt_stats* stats) {
    Range range_("bt_adjoint");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built && ctx->mat.done, BT_ERR_STATE, "bt_adjoint: mesh not assembled");
        BT_REQUIRE(!bt::strong_active(ctx), BT_ERR_STATE, "bt_adjoint: not defined with the strong pseudo-periodic form");
        BT_REQUIRE(ctx->sched.set, BT_ERR_STATE, "bt_adjoint: no schedule");
        BT_REQUIRE(gdir && signal_out, BT_ERR_INVALID, "bt_adjoint: bad arguments");
        BT_REQUIRE(std::isfinite(q) && std::isfinite(gdir[0]) && std::isfinite(gdir[1]) && std::isfinite(gdir[2]),
                   BT_ERR_INVALID, "bt_adjoint: q and gdir must be finite");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_adjoint: rtol must be > 0 and max_iterations >= 1");
        if (u0)
            for (int64_t v = 0; v < ctx->mesh.n_v; ++v)
                BT_REQUIRE(std::isfinite(u0[v]), BT_ERR_INVALID, "bt_adjoint: u0 must be finite");
        use_device(ctx);
        bt::adjoint_fp64(ctx, q, gdir, sequence, u0, rtol, max_iterations, checkpoint_stride, signal_out, dS_dD,
                         dS_dinvT2, dS_dkappa, stats);
        ctx->last_precision = -1;
    });
}

int bt_adjoint_cells(bt_ctx* ctx, double q, const double* gdir, int32_t sequence, const double* u0, double rtol,
                     int32_t max_iterations, int32_t checkpoint_stride, double* signal_out, double* dS_dD_cell,
                     double* dS_dinvT2_cell, double* dS_dkappa, bt_stats* stats) {
    Range range_("bt_adjoint_cells");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built && ctx->mat.done, BT_ERR_STATE, "bt_adjoint_cells: mesh not assembled");
        BT_REQUIRE(!bt::strong_active(ctx), BT_ERR_STATE,
                   "bt_adjoint_cells: not defined with the strong pseudo-periodic form");
        BT_REQUIRE(ctx->sched.set, BT_ERR_STATE, "bt_adjoint_cells: no schedule");
        BT_REQUIRE(gdir && signal_out, BT_ERR_INVALID, "bt_adjoint_cells: bad arguments");
        BT_REQUIRE(std::isfinite(q) && std::isfinite(gdir[0]) && std::isfinite(gdir[1]) && std::isfinite(gdir[2]),
                   BT_ERR_INVALID, "bt_adjoint_cells: q and gdir must be finite");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_adjoint_cells: rtol must be > 0 and max_iterations >= 1");
        if (u0)
            for (int64_t v = 0; v < ctx->mesh.n_v; ++v)
                BT_REQUIRE(std::isfinite(u0[v]), BT_ERR_INVALID, "bt_adjoint_cells: u0 must be finite");
        use_device(ctx);
        bt::adjoint_fp64(ctx, q, gdir, sequence, u0, rtol, max_iterations, checkpoint_stride, signal_out, nullptr,
                         nullptr, dS_dkappa, stats, dS_dD_cell, dS_dinvT2_cell);
        ctx->last_precision = -1;
    });
}

int bt_adjoint_batch(bt_ctx* ctx, int32_t n_signals, const double* q, const double* gdir, const int32_t* sequence,
                     double rtol, int32_t max_iterations, int32_t checkpoint_stride, double* signal_out,
                     double* dS_dD, double* dS_dinvT2, double* dS_dkappa, bt_stats* stats) {
    Range range_("bt_adjoint_batch");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built && ctx->mat.done, BT_ERR_STATE, "bt_adjoint_batch: mesh not assembled");
        BT_REQUIRE(!bt::strong_active(ctx), BT_ERR_STATE,
                   "bt_adjoint_batch: not defined with the strong pseudo-periodic form");
        BT_REQUIRE(ctx->sched.set, BT_ERR_STATE, "bt_adjoint_batch: no schedule");
        BT_REQUIRE(n_signals >= 1 && q && gdir && signal_out, BT_ERR_INVALID, "bt_adjoint_batch: bad arguments");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_adjoint_batch: rtol must be > 0 and max_iterations >= 1");
        for (int32_t i = 0; i < n_signals; ++i)
            BT_REQUIRE(std::isfinite(q[i]) && std::isfinite(gdir[3 * i]) && std::isfinite(gdir[3 * i + 1]) &&
                           std::isfinite(gdir[3 * i + 2]),
                       BT_ERR_INVALID, "bt_adjoint_batch: q and gdir must be finite");
        use_device(ctx);
        ctx->last_precision = -1;
        bt::adjoint_mixed(ctx, n_signals, q, gdir, sequence, rtol, max_iterations, checkpoint_stride, signal_out,
                          dS_dD, dS_dinvT2, dS_dkappa, stats);
    });
}

int bt_adjoint_batch_cells(bt_ctx* ctx, int32_t n_signals, const double* q, const double* gdir,
                           const int32_t* sequence, const double* weights, double rtol, int32_t max_iterations,
                           int32_t checkpoint_stride, double* signal_out, double* dS_dD_cell, double* dS_dinvT2_cell,
                           double* dS_dkappa, bt_stats* stats) {
    Range range_("bt_adjoint_batch_cells");
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mesh.built && ctx->mat.done, BT_ERR_STATE, "bt_adjoint_batch_cells: mesh not assembled");
        BT_REQUIRE(!bt::strong_active(ctx), BT_ERR_STATE,
                   "bt_adjoint_batch_cells: not defined with the strong pseudo-periodic form");
        BT_REQUIRE(ctx->sched.set, BT_ERR_STATE, "bt_adjoint_batch_cells: no schedule");
        BT_REQUIRE(n_signals >= 1 && q && gdir && weights && signal_out, BT_ERR_INVALID,
                   "bt_adjoint_batch_cells: bad arguments");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_adjoint_batch_cells: rtol must be > 0 and max_iterations >= 1");
        for (int32_t i = 0; i < n_signals; ++i)
            BT_REQUIRE(std::isfinite(q[i]) && std::isfinite(gdir[3 * i]) && std::isfinite(gdir[3 * i + 1]) &&
                           std::isfinite(gdir[3 * i + 2]) && std::isfinite(weights[i]),
                       BT_ERR_INVALID, "bt_adjoint_batch_cells: q, gdir and weights must be finite");
        use_device(ctx);
        ctx->last_precision = -1;
        bt::adjoint_mixed(ctx, n_signals, q, gdir, sequence, rtol, max_iterations, checkpoint_stride, signal_out,
                          nullptr, nullptr, dS_dkappa, stats, weights, dS_dD_cell, dS_dinvT2_cell);
    });
}

int bt_adjoint_multi(bt_ctx* const* contexts, int32_t n_meshes, const int32_t* n_signals, const double* q,
                     const double* gdir, const int32_t* sequence, double rtol, int32_t max_iterations,
                     int32_t checkpoint_stride, double* signal_out, double* dS_dD, double* dS_dinvT2,
                     double* dS_dkappa, bt_stats* stats) {
    Range range_("bt_adjoint_multi");
    if (!contexts || n_meshes < 1 || !contexts[0]) return BT_ERR_INVALID;
    bt_ctx* c0 = contexts[0];
    return guarded(c0, [&] {
        BT_REQUIRE(n_meshes <= 64 && n_signals && q && gdir && signal_out, BT_ERR_INVALID,
                   "bt_adjoint_multi: bad arguments (at most 64 meshes)");
        BT_REQUIRE(std::isfinite(rtol) && rtol > 0.0 && max_iterations >= 1, BT_ERR_INVALID,
                   "bt_adjoint_multi: rtol must be > 0 and max_iterations >= 1");
        int64_t total = 0;
        for (int32_t m = 0; m < n_meshes; ++m) {
            bt_ctx* c = contexts[m];
            BT_REQUIRE(c != nullptr, BT_ERR_INVALID, "bt_adjoint_multi: null context");
            for (int32_t j = 0; j < m; ++j)
                BT_REQUIRE(contexts[j] != c, BT_ERR_INVALID, "bt_adjoint_multi: a context is listed twice");
            BT_REQUIRE(c->device == c0->device, BT_ERR_INVALID, "bt_adjoint_multi: contexts on different devices");
            BT_REQUIRE(c->mesh.built && c->mat.done && c->sched.set, BT_ERR_STATE,
                       "bt_adjoint_multi: every mesh needs bt_assemble and bt_set_schedule");
            BT_REQUIRE(n_signals[m] >= 1 && n_signals[m] <= 256, BT_ERR_INVALID,
                       "bt_adjoint_multi: 1..256 signals per mesh");
            BT_REQUIRE(!bt::strong_active(c), BT_ERR_STATE,
                       "bt_adjoint_multi: not defined with the strong pseudo-periodic form");
            total += n_signals[m];
        }
        for (int64_t i = 0; i < total; ++i) {
            BT_REQUIRE(std::isfinite(q[i]) && std::isfinite(gdir[3 * i]) && std::isfinite(gdir[3 * i + 1]) &&
                           std::isfinite(gdir[3 * i + 2]),
                       BT_ERR_INVALID, "bt_adjoint_multi: q and gradient directions must be finite");
            if (sequence) {
                int64_t acc = 0;
                int32_t m = 0;
                while (acc + n_signals[m] <= i) acc += n_signals[m++];
                BT_REQUIRE(sequence[i] >= 0 && sequence[i] < contexts[m]->sched.n_seq, BT_ERR_INVALID,
                           "bt_adjoint_multi: sequence index out of range");
            }
        }
        use_device(c0);
        for (int32_t m = 0; m < n_meshes; ++m) contexts[m]->last_precision = -1;
        bt::adjoint_mixed_multi(contexts, n_meshes, n_signals, q, gdir, sequence, rtol, max_iterations,
                                checkpoint_stride, signal_out, dS_dD, dS_dinvT2, dS_dkappa, stats);
    });
}

int bt_set_option(bt_ctx* ctx, const char* key, double value) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(key && std::isfinite(value), BT_ERR_INVALID, "bt_set_option: bad key or value");
        const std::string k(key);
        const int iv = (int)value;
        if (k == "mixed.lanes_per_row") {
            BT_REQUIRE(iv == 0 || iv == 1 || iv == 2 || iv == 4 || iv == 8 || iv == 16 || iv == 32, BT_ERR_INVALID,
                       "mixed.lanes_per_row must be 0 or a power of two <= 32");
            ctx->opt_mixed_lpr = iv > 0 ? iv : -1;
            bt::reset_tuning_mixed(ctx);
        } else if (k == "mixed.blocks_per_sm") {
            BT_REQUIRE(iv >= 0 && iv <= 8, BT_ERR_INVALID, "mixed.blocks_per_sm must be in [0, 8]");
            ctx->opt_mixed_blocks_per_sm = iv > 0 ? iv : -1;
            bt::reset_tuning_mixed(ctx);
        } else if (k == "mixed.max_sweeps") {
            BT_REQUIRE(iv >= 1 && iv <= 64, BT_ERR_INVALID, "mixed.max_sweeps must be in [1, 64]");
            ctx->opt_mixed_max_sweeps = iv;
        } else if (k == "mixed.eps_first") {
            BT_REQUIRE(value > 0.0 && value < 1.0, BT_ERR_INVALID, "mixed.eps_first must be in (0, 1)");
            ctx->opt_mixed_eps_first = value;
        } else if (k == "mixed.eps_next") {
            BT_REQUIRE(value > 0.0 && value < 1.0, BT_ERR_INVALID, "mixed.eps_next must be in (0, 1)");
            ctx->opt_mixed_eps_next = value;
        } else if (k == "mixed.blocked_rows") {
            BT_REQUIRE(iv >= -1 && iv <= 1, BT_ERR_INVALID, "mixed.blocked_rows must be -1 (tune), 0 or 1");
            ctx->opt_mixed_blocked = iv;
            bt::reset_tuning_mixed(ctx);
        } else if (k == "mixed.reduce") {
            BT_REQUIRE(iv >= -1 && iv <= 1, BT_ERR_INVALID, "mixed.reduce must be -1 (by size), 0 or 1");
            ctx->opt_mixed_reduce = iv;
            bt::reset_tuning_mixed(ctx);
        } else if (k == "mixed.divergence") {
            BT_REQUIRE(value >= 1.0, BT_ERR_INVALID, "mixed.divergence must be >= 1");
            ctx->opt_mixed_growth2 = value * value;
        } else if (k == "mixed.extrapolate") {
            BT_REQUIRE(iv >= 0 && iv <= 4, BT_ERR_INVALID, "mixed.extrapolate must be in [0, 4]");
            ctx->opt_mixed_extrapolate = iv;
        } else if (k == "mixed.inner_reductions") {
            BT_REQUIRE(iv == 1 || iv == 2, BT_ERR_INVALID, "mixed.inner_reductions must be 1 or 2");
            ctx->opt_mixed_inner = iv;
            bt::reset_tuning_mixed(ctx);
        } else if (k == "strong.batch") {
            BT_REQUIRE(iv == 0 || iv == 1, BT_ERR_INVALID, "strong.batch must be 0 or 1");
            ctx->opt_strong_batch = iv;
        } else if (k == "mixed.sort_signals") {
            BT_REQUIRE(iv == 0 || iv == 1, BT_ERR_INVALID, "mixed.sort_signals must be 0 or 1");
            ctx->opt_mixed_sort = iv;
        } else if (k == "fp64.extrapolate") {
            BT_REQUIRE(iv >= 0 && iv <= 4, BT_ERR_INVALID, "fp64.extrapolate must be in [0, 4]");
            ctx->opt_fp64_extrapolate = iv;
        } else if (k == "fp64.pair_signals") {
            BT_REQUIRE(iv >= 0 && iv <= 2, BT_ERR_INVALID, "fp64.pair_signals must be 0, 1 or 2");
            ctx->opt_fp64_pair = iv;
        } else if (k == "fp64.blocks_per_sm") {
            BT_REQUIRE(iv >= -1 && iv <= 8, BT_ERR_INVALID, "fp64.blocks_per_sm must be in [-1, 8]");
            ctx->opt_fp64_blocks_per_sm = iv;
        } else if (k == "wait.limit_ns") {
            BT_REQUIRE(value >= 1e4 && value <= 6e10, BT_ERR_INVALID, "wait.limit_ns must be in [1e4, 6e10]");
            ctx->opt_wait_ns = (unsigned long long)value;
        } else if (k == "test.stall_first_wait") {
            ctx->opt_stall_first_wait = iv ? 1 : 0;
        } else {
            throw bt::Error(BT_ERR_INVALID, "bt_set_option: unknown key " + k);
        }
    });
}

int bt_get_csr(bt_ctx* ctx, int32_t* row_ptr, int32_t* col) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Mesh& m = ctx->mesh;
        BT_REQUIRE(m.built, BT_ERR_STATE, "bt_get_csr: no mesh");
        use_device(ctx);
        if (row_ptr) m.row_ptr.download(row_ptr, m.n_dofs + 1, ctx->stream);
        if (col) m.col.download(col, m.nnz, ctx->stream);
        BT_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int bt_get_matrix(bt_ctx* ctx, int32_t which, double* values) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(ctx->mat.done, BT_ERR_STATE, "bt_get_matrix: not assembled");
        BT_REQUIRE(values, BT_ERR_INVALID, "bt_get_matrix: NULL output");
        use_device(ctx);
        const bt::DevBuf<double>* src[] = {&ctx->mat.M, &ctx->mat.K, &ctx->mat.T, &ctx->mat.R,
                                           &ctx->mat.Jx, &ctx->mat.Jy, &ctx->mat.Jz};
        BT_REQUIRE(which >= 0 && which < 7, BT_ERR_INVALID, "bt_get_matrix: unknown matrix");
        src[which]->download(values, ctx->mesh.nnz, ctx->stream);
        BT_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int bt_get_dofs(bt_ctx* ctx, int32_t* dof_vertex, int32_t* dof_compartment, double* weights) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Mesh& m = ctx->mesh;
        BT_REQUIRE(m.built, BT_ERR_STATE, "bt_get_dofs: no mesh");
        use_device(ctx);
        if (dof_vertex) m.dof_vertex.download(dof_vertex, m.n_dofs, ctx->stream);
        if (dof_compartment) m.dof_comp.download(dof_compartment, m.n_dofs, ctx->stream);
        if (weights) {
            BT_REQUIRE(ctx->mat.done, BT_ERR_STATE, "bt_get_dofs: weights need bt_assemble");
            ctx->mat.w.download(weights, m.n_dofs, ctx->stream);
        }
        BT_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int bt_get_colouring(bt_ctx* ctx, int32_t* cell_colour) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        const bt::Mesh& m = ctx->mesh;
        BT_REQUIRE(m.built && cell_colour, BT_ERR_INVALID, "bt_get_colouring: no mesh or NULL output");
        use_device(ctx);
        m.colour.download(cell_colour, m.n_t, ctx->stream);
        BT_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int bt_get_solution(bt_ctx* ctx, int32_t index, double* u) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(u, BT_ERR_INVALID, "bt_get_solution: NULL output");
        use_device(ctx);
        BT_REQUIRE(ctx->last_precision >= 0, BT_ERR_STATE, "bt_get_solution: no solve yet");
        if (ctx->last_strong)
            bt::get_solution_strong(ctx, index, u);
        else if (ctx->last_precision == BT_PRECISION_MIXED)
            bt::get_solution_mixed(ctx, index, u);
        else
            bt::get_solution_fp64(ctx, index, u);
    });
}

int bt_get_iterations(bt_ctx* ctx, int32_t* iters, int64_t capacity) {
    if (!ctx) return BT_ERR_INVALID;
    return guarded(ctx, [&] {
        BT_REQUIRE(iters, BT_ERR_INVALID, "bt_get_iterations: NULL output");
        BT_REQUIRE(capacity >= (int64_t)ctx->last_iters.size(), BT_ERR_INVALID,
                   "bt_get_iterations: buffer smaller than n_signals*n_steps");
        std::memcpy(iters, ctx->last_iters.data(), ctx->last_iters.size() * sizeof(int32_t));
    });
}

}  // extern "C"
