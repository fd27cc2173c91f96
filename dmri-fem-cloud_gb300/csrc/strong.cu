// Strong pseudo-periodic boundaries: the constrained periodic space and a
// persistent FP64 Jacobi-BiCGSTAB stepper.
//
// Reference: mydomain.IsDomainPeriodic = True with PeriodicDir set.
//   * MyFunctionSpaces (DmriFemLib.py:453-486) builds the function space with
//     constrained_domain = PeriodicBD (DmriFemLib.py:325-378).  DOLFIN pairs every
//     vertex of an exterior facet that is not `inside` the target boundary with
//     the vertex at map(x) when map(x) is `inside`; inside() is the whole min
//     face of each periodic direction (tolerance 1e-2 hmin), map() shifts x by
//     the box length along the first periodic direction whose max face holds x.
//     Nothing is chained, so with several periodic directions the edge columns
//     (xmax, ymin) and (xmin, ymin) stay separate dofs, as in the reference.
//   * ThetaMethodF_sBC1c/2c and ThetaMethodL_sBC1c/2c (DmriFemLib.py:148-238):
//     FuncF_sBC in the cells, outer_interface on every exterior facet and
//     inner_interface on compartment interfaces (normal of the phase-0 side,
//     avg(D) on both sides), with ift = itime_profile(t) in F and
//     itime_profile(tp) in L, and +theta on the explicit operator
//     (DmriFemLib.py:878-915).
// On one complex dof per (vertex class, compartment) pair the step reads
//     (M/k + theta (S + q^2 F^2 M_D + i q F E)) u_{n+1}
//         = (M/k - theta (S + q^2 Fp^2 M_D + i q Fp E)) u_n,
//     S = K + T + R,  (M_D)_ij = int (g.D g) phi_i phi_j,
//     E = C - B,  C_ij = int 2 (D g).grad phi_j phi_i,
//     B_ij = int_{boundary of the dof's compartment} (Dbar g).n phi_i phi_j.
// E is linear and M_D quadratic in g, so the set-up stores E_k (k = x, y, z)
// and the six components of M_D per stored entry, and a pack kernel forms
// theta q E_g and theta q^2 (M_D)_g per signal.  The operator is neither complex
// symmetric nor Hermitian in general (it is Hermitian for one compartment of
// constant D), so the linear solver is BiCGSTAB (van der Vorst 1992) with the
// conjugated inner product and the Jacobi preconditioner, as PETSc's BCGS.
//
// The reference's phase-blind outer term also acts on the dead rows of the
// other compartment at interface vertices on the exterior boundary.  It
// cancels between opposite periodic faces when the compartments are periodic
// (checked here: a folded vertex must touch the compartments of its master)
// and vanishes where (D g).n = 0; the set-up records the directions in which
// it does not vanish on some facet, and a solve whose g has a component there
// is refused, since the duplicated-node system would leave that term out.
//
// The set-up (periodic pairing, folded sparsity, first-order and boundary
// integrals) runs on the host once per mesh and coefficient set, like the
// weak form's; the time loop is one cooperative launch per signal.
#include "bt_common.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <unordered_map>
#include <vector>

namespace bt {

constexpr int kThreadsS = 256;
constexpr int kRedS = 4;   // doubles per block partial

struct Strong {
    int32_t dir[3] = {0, 0, 0};
    bool on = false;
    int64_t built_version = -1;
    int64_t n = 0, nnz = 0, n_classes = 0;
    bool excess_dir[3] = {false, false, false};
    std::vector<int32_t> fold;              // unfolded dof -> folded dof
    DevBuf<int32_t> row_ptr, col, diag, rcomp, u0_vertex;
    DevBuf<double> m, s, md6, e3, w;        // per entry: M, S, 6 x M_D, 3 x E; per row: signal weight
    // per-signal workspace
    int32_t nblocks = 0;
    DevBuf<double> are, mdg, eg;            // per entry: M/k + theta S, theta q^2 (M_D)_g, theta q E_g
    DevBuf<double> Fn, Fo;                  // F(t), F(tp) per step
    DevBuf<double2> u[3], r, rh, p, v, sv, t, y, z, dinv, ac;
    DevBuf<double> partials, out, relres;
    DevBuf<unsigned> bar;
    DevBuf<int> status;
    DevBuf<int32_t> iters;
    DevBuf<double2> saved;
    int32_t saved_nsig = 0;
    // batched stepper (several signals of one gradient direction): vectors [row][32]
    int32_t mblocks = 0;
    DevBuf<double2> mu[3], mr, mrh, mp, mv, ms, mt, my, mz, mdinv;
    DevBuf<double> mq, mg, mFn, mFo, mpart, mfin, mout, mrel;
};

namespace {

inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Hash grid of master vertices, cells of side h (several times the match
// tolerance), queried over the 27 neighbouring cells.
struct PointIndex {
    double h = 1.0, lo[3] = {0, 0, 0};
    std::unordered_map<long long, std::vector<int32_t>> cells;
    long long key(long long i, long long j, long long k) const {
        return (i * 2097143LL + j) * 2097169LL + k;
    }
    void add(const double* x, int32_t v) {
        cells[key(llround((x[0] - lo[0]) / h), llround((x[1] - lo[1]) / h), llround((x[2] - lo[2]) / h))]
            .push_back(v);
    }
    int32_t find(const std::vector<double>& xyz, const double* y, double tol) const {
        const long long i0 = llround((y[0] - lo[0]) / h), j0 = llround((y[1] - lo[1]) / h),
                        k0 = llround((y[2] - lo[2]) / h);
        int32_t best = -1;
        double bd = tol;
        for (long long i = i0 - 1; i <= i0 + 1; ++i)
            for (long long j = j0 - 1; j <= j0 + 1; ++j)
                for (long long k = k0 - 1; k <= k0 + 1; ++k) {
                    auto it = cells.find(key(i, j, k));
                    if (it == cells.end()) continue;
                    for (int32_t v : it->second) {
                        double d = 0.0;
                        for (int a = 0; a < 3; ++a) d = std::max(d, std::fabs(xyz[3 * (size_t)v + a] - y[a]));
                        if (d <= bd) {
                            bd = d;
                            best = v;
                        }
                    }
                }
        return best;
    }
};

// 3x3 symmetric D of cell t
inline void cell_D(const std::vector<double>& Dr, const std::vector<double>& Dc, const std::vector<int32_t>& region,
                   int64_t t, double D[3][3]) {
    if (!Dc.empty()) {
        const double* d = Dc.data() + (size_t)t * 6;
        D[0][0] = d[0]; D[1][1] = d[1]; D[2][2] = d[2];
        D[0][1] = D[1][0] = d[3];
        D[0][2] = D[2][0] = d[4];
        D[1][2] = D[2][1] = d[5];
    } else {
        const double s = Dr[region[t]];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) D[r][c] = (r == c) ? s : 0.0;
    }
}

}  // namespace

// ----------------------------------------------------------------- set-up --
static void build_strong(bt_ctx* ctx, Strong& P) {
    Mesh& m = ctx->mesh;
    Assembled& A = ctx->mat;
    Coeffs& cf = ctx->coeffs;
    cudaStream_t s = ctx->stream;
    const int64_t n_v = m.n_v, n_t = m.n_t, nc = m.n_comp, n = m.n_dofs, nnz = m.nnz;
    BT_REQUIRE(nc <= 2, BT_ERR_INVALID,
               "strong pseudo-periodic form: at most two compartments (the reference's inner_interface)");
    std::vector<double> xyz((size_t)n_v * 3), hM((size_t)nnz), hK((size_t)nnz), hT((size_t)nnz), hR((size_t)nnz),
        hw((size_t)n), Dr((size_t)m.n_regions), Dc;
    std::vector<int32_t> tets((size_t)n_t * 4), comp((size_t)n_t), region((size_t)n_t), nbr((size_t)n_t * 4),
        dof_of((size_t)n_v * nc), rp((size_t)n + 1), col((size_t)nnz), dvert((size_t)n), dcomp((size_t)n);
    m.xyz.download(xyz.data(), xyz.size(), s);
    m.tets.download(tets.data(), tets.size(), s);
    m.comp.download(comp.data(), comp.size(), s);
    m.region.download(region.data(), region.size(), s);
    m.nbr.download(nbr.data(), nbr.size(), s);
    m.dof_of.download(dof_of.data(), dof_of.size(), s);
    m.row_ptr.download(rp.data(), rp.size(), s);
    m.col.download(col.data(), col.size(), s);
    m.dof_vertex.download(dvert.data(), dvert.size(), s);
    m.dof_comp.download(dcomp.data(), dcomp.size(), s);
    A.M.download(hM.data(), hM.size(), s);
    A.K.download(hK.data(), hK.size(), s);
    A.T.download(hT.data(), hT.size(), s);
    A.R.download(hR.data(), hR.size(), s);
    A.w.download(hw.data(), hw.size(), s);
    cf.D_region.download(Dr.data(), Dr.size(), s);
    if (cf.has_cell_D) {
        Dc.resize((size_t)n_t * 6);
        cf.D_cell.download(Dc.data(), Dc.size(), s);
    }
    BT_CUDA(cudaStreamSynchronize(s));

    // box, hmin (smallest cell diameter), tolerance of PeriodicBD
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t v = 0; v < n_v; ++v)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], xyz[3 * v + d]);
            hi[d] = std::max(hi[d], xyz[3 * v + d]);
        }
    double hmin = 1e300;
    for (int64_t t = 0; t < n_t; ++t) {
        double h2 = 0.0;
        for (int a = 0; a < 4; ++a)
            for (int b = a + 1; b < 4; ++b) {
                double e2 = 0.0;
                for (int d = 0; d < 3; ++d) {
                    const double dd = xyz[3 * (size_t)tets[4 * t + a] + d] - xyz[3 * (size_t)tets[4 * t + b] + d];
                    e2 += dd * dd;
                }
                h2 = std::max(h2, e2);
            }
        hmin = std::min(hmin, std::sqrt(h2));
    }
    BT_REQUIRE(hmin > 0.0 && std::isfinite(hmin), BT_ERR_INVALID, "strong periodic set-up: degenerate mesh");
    const double tol = 1e-2 * hmin;
    const double match_tol = 1e-6 * hmin;
    const int* dir = P.dir;
    auto inside = [&](const double* x) {
        for (int d = 0; d < 3; ++d)
            if (dir[d] && std::fabs(x[d] - lo[d]) < tol) return true;
        return false;
    };

    // vertices of exterior facets; masters are those inside the target boundary
    std::vector<char> bnd((size_t)n_v, 0);
    for (int64_t t = 0; t < n_t; ++t)
        for (int a = 0; a < 4; ++a)
            if (nbr[4 * t + a] < 0)
                for (int b = 0; b < 4; ++b)
                    if (b != a) bnd[tets[4 * t + b]] = 1;
    PointIndex idx;
    idx.h = 4.0 * match_tol;
    for (int d = 0; d < 3; ++d) idx.lo[d] = lo[d];
    for (int64_t v = 0; v < n_v; ++v)
        if (bnd[v] && inside(&xyz[3 * v])) idx.add(&xyz[3 * v], (int32_t)v);
    std::vector<int32_t> master((size_t)n_v);
    for (int64_t v = 0; v < n_v; ++v) master[v] = (int32_t)v;
    for (int64_t v = 0; v < n_v; ++v) {
        if (!bnd[v]) continue;
        const double* x = &xyz[3 * v];
        if (inside(x)) continue;
        double y[3] = {x[0], x[1], x[2]};
        bool mapped = false;
        for (int d = 0; d < 3 && !mapped; ++d)
            if (dir[d] && std::fabs(x[d] - hi[d]) < tol) {
                y[d] = x[d] - (hi[d] - lo[d]);
                mapped = true;
            }
        if (!mapped || !inside(y)) continue;
        const int32_t mv = idx.find(xyz, y, match_tol);
        BT_REQUIRE(mv >= 0, BT_ERR_INVALID,
                   "strong periodic set-up: a vertex on a periodic face has no vertex at its image (mesh not "
                   "periodic)");
        master[v] = mv;
    }
    // compartments touching each vertex; a slave must touch those of its master
    std::vector<unsigned> touch((size_t)n_v, 0u);
    for (int64_t t = 0; t < n_t; ++t)
        for (int a = 0; a < 4; ++a) touch[tets[4 * t + a]] |= 1u << comp[t];
    for (int64_t v = 0; v < n_v; ++v)
        BT_REQUIRE(touch[v] == touch[master[v]], BT_ERR_INVALID,
                   "strong periodic set-up: compartments are not periodic (a vertex on a periodic face touches "
                   "other compartments than its image)");

    // folded dofs: masters in unfolded order, slaves take their master's
    std::vector<int32_t> fold((size_t)n, -1), fvert, fcomp;
    for (int64_t i = 0; i < n; ++i)
        if (master[dvert[i]] == dvert[i]) {
            fold[i] = (int32_t)fvert.size();
            fvert.push_back(dvert[i]);
            fcomp.push_back(dcomp[i]);
        }
    for (int64_t i = 0; i < n; ++i)
        if (fold[i] < 0) {
            const int32_t j = dof_of[(size_t)master[dvert[i]] * nc + dcomp[i]];
            BT_REQUIRE(j >= 0 && fold[j] >= 0, BT_ERR_INVALID, "strong periodic set-up: master dof missing");
            fold[i] = fold[j];
        }
    const int64_t nf = (int64_t)fvert.size();

    // folded sparsity: the images of the stored pairs, sorted per row
    std::vector<std::vector<int32_t>> rows((size_t)nf);
    for (int64_t i = 0; i < n; ++i)
        for (int32_t e = rp[i]; e < rp[i + 1]; ++e) rows[fold[i]].push_back(fold[col[e]]);
    std::vector<int32_t> frp((size_t)nf + 1, 0), fcol;
    for (int64_t i = 0; i < nf; ++i) {
        auto& r = rows[i];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        fcol.insert(fcol.end(), r.begin(), r.end());
        frp[i + 1] = (int32_t)fcol.size();
        std::vector<int32_t>().swap(r);
    }
    const int64_t fnnz = (int64_t)fcol.size();
    BT_REQUIRE(fnnz < (int64_t)INT32_MAX, BT_ERR_INVALID, "strong periodic set-up: too many entries");
    auto pos = [&](int32_t i, int32_t j) -> int64_t {
        const int32_t* b = fcol.data() + frp[i];
        const int32_t* e = fcol.data() + frp[i + 1];
        const int32_t* it = std::lower_bound(b, e, j);
        BT_REQUIRE(it != e && *it == j, BT_ERR_INVALID, "strong periodic set-up: pair outside the sparsity");
        return (int64_t)(it - fcol.data());
    };
    std::vector<double> fm((size_t)fnnz, 0.0), fs((size_t)fnnz, 0.0), fmd((size_t)fnnz * 6, 0.0),
        fe((size_t)fnnz * 3, 0.0), fw((size_t)nf, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        fw[fold[i]] += hw[i];
        for (int32_t e = rp[i]; e < rp[i + 1]; ++e) {
            const int64_t p = pos(fold[i], fold[col[e]]);
            fm[p] += hM[e];
            fs[p] += hK[e] + hT[e] + hR[e];
        }
    }

    // cells: C_k (first-order term per unit g_k) and the six components of M_D
    for (int64_t t = 0; t < n_t; ++t) {
        const int32_t* tv = &tets[4 * t];
        const int c = comp[t];
        double X[4][3];
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d) X[a][d] = xyz[3 * (size_t)tv[a] + d];
        double E[3][3];
        for (int r = 0; r < 3; ++r)
            for (int d = 0; d < 3; ++d) E[r][d] = X[r + 1][d] - X[0][d];
        const double det = E[0][0] * (E[1][1] * E[2][2] - E[1][2] * E[2][1]) -
                           E[0][1] * (E[1][0] * E[2][2] - E[1][2] * E[2][0]) +
                           E[0][2] * (E[1][0] * E[2][1] - E[1][1] * E[2][0]);
        const double vol = std::fabs(det) / 6.0;
        // gradients of the barycentric coordinates: rows of E^-T
        double G[4][3];
        double c0[3], c1[3], c2[3];
        cross3(E[1], E[2], c0);
        cross3(E[2], E[0], c1);
        cross3(E[0], E[1], c2);
        for (int d = 0; d < 3; ++d) {
            G[1][d] = c0[d] / det;
            G[2][d] = c1[d] / det;
            G[3][d] = c2[d] / det;
            G[0][d] = -(G[1][d] + G[2][d] + G[3][d]);
        }
        double D[3][3];
        cell_D(Dr, Dc, region, t, D);
        int32_t fd[4];
        for (int a = 0; a < 4; ++a) fd[a] = fold[dof_of[(size_t)tv[a] * nc + c]];
        const double mdc[6] = {D[0][0], D[1][1], D[2][2], 2.0 * D[0][1], 2.0 * D[0][2], 2.0 * D[1][2]};
        for (int j = 0; j < 4; ++j) {
            double DG[3];
            for (int k = 0; k < 3; ++k) DG[k] = D[k][0] * G[j][0] + D[k][1] * G[j][1] + D[k][2] * G[j][2];
            for (int i = 0; i < 4; ++i) {
                const int64_t p = pos(fd[i], fd[j]);
                for (int k = 0; k < 3; ++k) fe[3 * (size_t)p + k] += 0.5 * vol * DG[k];   // (vol/4) * 2 (D grad phi_j)_k
                const double mass = vol / 20.0 * (i == j ? 2.0 : 1.0);
                for (int k = 0; k < 6; ++k) fmd[6 * (size_t)p + k] += mass * mdc[k];
            }
        }
    }

    // facets: outward normal of cell t at the face opposite local vertex a
    auto facet = [&](int64_t t, int a, int32_t fv[3], double nrm[3], double& area) {
        const int32_t* tv = &tets[4 * t];
        int k = 0;
        for (int b = 0; b < 4; ++b)
            if (b != a) fv[k++] = tv[b];
        double e1[3], e2[3], cr[3], off[3];
        for (int d = 0; d < 3; ++d) {
            e1[d] = xyz[3 * (size_t)fv[1] + d] - xyz[3 * (size_t)fv[0] + d];
            e2[d] = xyz[3 * (size_t)fv[2] + d] - xyz[3 * (size_t)fv[0] + d];
            off[d] = xyz[3 * (size_t)fv[0] + d] - xyz[3 * (size_t)tv[a] + d];
        }
        cross3(e1, e2, cr);
        const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        area = 0.5 * len;
        const double sg = (cr[0] * off[0] + cr[1] * off[1] + cr[2] * off[2]) >= 0.0 ? 1.0 : -1.0;
        for (int d = 0; d < 3; ++d) nrm[d] = sg * cr[d] / len;
    };
    // phase-blind remainder of the reference's outer term on the other compartment
    // of interface vertices: (row class, compartment, column class) -> coefficient per g_k
    std::map<std::array<int64_t, 3>, std::array<double, 3>> excess;
    double dscale = 0.0;
    for (int64_t t = 0; t < n_t; ++t)
        for (int a = 0; a < 4; ++a) {
            const int32_t tn = nbr[4 * t + a];
            if (tn >= 0 && (comp[tn] == comp[t] || tn < t)) continue;
            int32_t fv[3];
            double nrm[3], area;
            facet(t, a, fv, nrm, area);
            if (tn < 0) {
                // exterior facet: outer_interface on the cell's compartment, -(D g).n phi phi in E
                const int c = comp[t];
                double D[3][3];
                cell_D(Dr, Dc, region, t, D);
                double Dn[3];
                for (int k = 0; k < 3; ++k) Dn[k] = D[k][0] * nrm[0] + D[k][1] * nrm[1] + D[k][2] * nrm[2];
                for (int k = 0; k < 3; ++k) dscale = std::max(dscale, std::fabs(Dn[k]) * area);
                int32_t fd[3];
                for (int b = 0; b < 3; ++b) fd[b] = fold[dof_of[(size_t)fv[b] * nc + c]];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        const double mass = area / 12.0 * (i == j ? 2.0 : 1.0);
                        const int64_t p = pos(fd[i], fd[j]);
                        for (int k = 0; k < 3; ++k) fe[3 * (size_t)p + k] -= Dn[k] * mass;
                    }
                for (int i = 0; i < 3; ++i)
                    for (int oc = 0; oc < nc; ++oc) {
                        if (oc == c || !(touch[fv[i]] & (1u << oc))) continue;
                        for (int j = 0; j < 3; ++j) {
                            const double mass = area / 12.0 * (i == j ? 2.0 : 1.0);
                            auto& ex = excess[{(int64_t)master[fv[i]], (int64_t)oc, (int64_t)master[fv[j]]}];
                            for (int k = 0; k < 3; ++k) ex[k] += Dn[k] * mass;
                        }
                    }
            } else {
                // compartment interface: inner_interface, -(Dbar g).n0 phi phi on the
                // phase-0 side and +(Dbar g).n0 phi phi on the other
                const int64_t t0 = comp[t] == 0 ? t : (int64_t)tn;
                const int64_t t1 = comp[t] == 0 ? (int64_t)tn : t;
                const double sg = (t0 == t) ? 1.0 : -1.0;   // nrm is the outward normal of t
                double D0[3][3], D1[3][3], Dn[3];
                cell_D(Dr, Dc, region, t0, D0);
                cell_D(Dr, Dc, region, t1, D1);
                for (int k = 0; k < 3; ++k) {
                    Dn[k] = 0.0;
                    for (int d = 0; d < 3; ++d) Dn[k] += 0.5 * (D0[k][d] + D1[k][d]) * sg * nrm[d];
                }
                for (int side = 0; side < 2; ++side) {
                    const int c = comp[side == 0 ? t0 : t1];
                    const double sgn = side == 0 ? -1.0 : 1.0;
                    int32_t fd[3];
                    for (int b = 0; b < 3; ++b) fd[b] = fold[dof_of[(size_t)fv[b] * nc + c]];
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) {
                            const double mass = area / 12.0 * (i == j ? 2.0 : 1.0);
                            const int64_t p = pos(fd[i], fd[j]);
                            for (int k = 0; k < 3; ++k) fe[3 * (size_t)p + k] += sgn * Dn[k] * mass;
                        }
                }
            }
        }
    for (int k = 0; k < 3; ++k) P.excess_dir[k] = false;
    for (const auto& kv : excess)
        for (int k = 0; k < 3; ++k)
            if (std::fabs(kv.second[k]) > 1e-10 * dscale) P.excess_dir[k] = true;

    std::vector<int32_t> fdiag((size_t)nf), u0v((size_t)nf);
    for (int64_t i = 0; i < nf; ++i) {
        fdiag[i] = (int32_t)pos((int32_t)i, (int32_t)i);
        u0v[i] = fvert[i];
    }
    P.n = nf;
    P.nnz = fnnz;
    P.n_classes = 0;
    for (int64_t v = 0; v < n_v; ++v) P.n_classes += master[v] == v;
    P.fold = fold;
    P.row_ptr.upload(frp.data(), frp.size(), s);
    P.col.upload(fcol.data(), fcol.size(), s);
    P.diag.upload(fdiag.data(), fdiag.size(), s);
    P.rcomp.upload(fcomp.data(), fcomp.size(), s);
    P.u0_vertex.upload(u0v.data(), u0v.size(), s);
    P.m.upload(fm.data(), fm.size(), s);
    P.s.upload(fs.data(), fs.size(), s);
    P.md6.upload(fmd.data(), fmd.size(), s);
    P.e3.upload(fe.data(), fe.size(), s);
    P.w.upload(fw.data(), fw.size(), s);
    BT_CUDA(cudaStreamSynchronize(s));
}

// -------------------------------------------------------------- kernels --
__global__ void k_sbc_pack(int64_t nnz, const double* __restrict__ m, const double* __restrict__ s,
                           const double* __restrict__ md6, const double* __restrict__ e3, double inv_k,
                           double theta, double q, double gx, double gy, double gz, double* __restrict__ are,
                           double* __restrict__ mdg, double* __restrict__ eg) {
    const double gg[6] = {gx * gx, gy * gy, gz * gz, gx * gy, gx * gz, gy * gz};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        are[e] = m[e] * inv_k + theta * s[e];
        double a = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) a += md6[6 * e + k] * gg[k];
        mdg[e] = theta * q * q * a;
        eg[e] = theta * q * (e3[3 * e] * gx + e3[3 * e + 1] * gy + e3[3 * e + 2] * gz);
    }
}

__global__ void k_sbc_init(int64_t n, const int32_t* __restrict__ u0_vertex, const double* __restrict__ u0,
                           double2* __restrict__ u) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        u[i] = make_double2(u0 ? u0[u0_vertex[i]] : 1.0, 0.0);
}

struct SbcArgs {
    int64_t n;
    const int32_t* __restrict__ row_ptr;
    const int32_t* __restrict__ col;
    const int32_t* __restrict__ diag;
    const int32_t* __restrict__ rcomp;
    const double* __restrict__ m;
    const double* __restrict__ are;
    const double* __restrict__ mdg;
    const double* __restrict__ eg;
    const double* __restrict__ w;
    const double* __restrict__ Fn;
    const double* __restrict__ Fo;
    double inv_k;
    double2* u0;              // three rotating solution levels u_{n-1}, u_n, u_{n+1}
    double2* u1;
    double2* u2;
    int32_t extrapolate;      // 1: initial guess 2 u_n - u_{n-1} from the second step on
    double2 *r, *rh, *p, *v, *sv, *t, *y, *z, *dinv;
    double2* ac;              // this step's A(F) = (A_re + F^2 M_D, F E) per stored entry
    double* partials;
    unsigned* bar;
    int* status;
    int32_t* iters;
    double* relres;
    double* out;
    int32_t n_steps, maxit, nc;
    double rtol2;
    unsigned long long wait_ns;
};

// conj(a) * b
__device__ __forceinline__ double2 cdotc(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// Sum of kRedS doubles over the grid: block partials into one of two alternating
// buffers, a barrier, then every block adds the partials in block order.
__device__ __forceinline__ bool sbc_reduce(double (&v)[kRedS], const SbcArgs& a, unsigned nb, unsigned& flip,
                                           unsigned& gen, double* sm) {
    block_sum<kRedS>(v, sm);
    double* P = a.partials + (size_t)(flip & 1u) * nb * kRedS;
    ++flip;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < kRedS; ++k) P[blockIdx.x * kRedS + k] = v[k];
    }
    if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return false;
    __shared__ double red[kRedS];
    grid_partials_sum<kRedS>(P, nb, red);
#pragma unroll
    for (int k = 0; k < kRedS; ++k) v[k] = red[k];
    __syncthreads();
    return true;
}

// Four lanes per row: y_i = sum_j (c0 * are + c1 * mdg + c2 * m + i c3 * eg)_ij x_j
// and, when kTwo, y2_i = sum_j (d0 * are + d1 * mdg + d2 * m + i d3 * eg)_ij x2_j with
// x2 = 2 x - xp when ext (else x); calls f(row, y_i, y2_i) on lane 0 of each row
// group (every lane of the warp runs the same iterations, for the shuffles).  x
// and xp are written inside the launch: plain coherent loads.
template <bool kTwo, typename F>
__device__ __forceinline__ void sbc_spmv(const SbcArgs& a, const double2* x, const double2* xp, bool ext,
                                         double c0, double c1, double c2, double c3, double d0, double d1,
                                         double d2, double d3, F&& f) {
    // with kTwo (phase R) the second coefficient set is A(F) = (d0 A_re + d1 M_D, d3 E), stored in ac
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int sub = lane & 3;
    for (int64_t base = gw * 8; base < a.n; base += nw * 8) {
        const int64_t row = base + (lane >> 2);
        double2 acc = make_double2(0.0, 0.0), acc2 = make_double2(0.0, 0.0);
        if (row < a.n) {
            const int32_t e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
            for (int32_t e = e0 + sub; e < e1; e += 4) {
                const double ar = a.are[e], md = a.mdg[e], mm = a.m[e], ev = a.eg[e];
                const double2 xv = x[a.col[e]];
                const double re = c0 * ar + c1 * md + c2 * mm, im = c3 * ev;
                acc.x += re * xv.x - im * xv.y;
                acc.y += re * xv.y + im * xv.x;
                if (kTwo) {
                    const double re2 = d0 * ar + d1 * md + d2 * mm, im2 = d3 * ev;
                    double2 x2 = xv;
                    if (ext) {
                        const double2 xo = xp[a.col[e]];
                        x2 = make_double2(2.0 * xv.x - xo.x, 2.0 * xv.y - xo.y);
                    }
                    acc2.x += re2 * x2.x - im2 * x2.y;
                    acc2.y += re2 * x2.y + im2 * x2.x;
                    a.ac[e] = make_double2(re2, im2);
                }
            }
        }
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
            if (kTwo) {
                acc2.x += __shfl_xor_sync(0xffffffffu, acc2.x, o);
                acc2.y += __shfl_xor_sync(0xffffffffu, acc2.y, o);
            }
        }
        if (row < a.n && sub == 0) f(row, acc, acc2);
    }
}

// Four lanes per row: y_i = sum_j ac_ij x_j with this step's stored A(F) values;
// calls f(row, y_i) on lane 0 of each row group.
template <typename F>
__device__ __forceinline__ void sbc_apply(const SbcArgs& a, const double2* x, F&& f) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int sub = lane & 3;
    for (int64_t base = gw * 8; base < a.n; base += nw * 8) {
        const int64_t row = base + (lane >> 2);
        double2 acc = make_double2(0.0, 0.0);
        if (row < a.n) {
            const int32_t e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
            for (int32_t e = e0 + sub; e < e1; e += 4) {
                const double2 m = a.ac[e];
                const double2 xv = x[a.col[e]];
                acc.x = fma(m.x, xv.x, fma(-m.y, xv.y, acc.x));
                acc.y = fma(m.x, xv.y, fma(m.y, xv.x, acc.y));
            }
        }
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        }
        if (row < a.n && sub == 0) f(row, acc);
    }
}

__global__ void __launch_bounds__(kThreadsS, 2) k_step_sbc(SbcArgs a) {
    __shared__ double sm[32 * kRedS];
    const unsigned nb = gridDim.x;
    unsigned gen = 0, flip = 0;
    const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nt = (int64_t)gridDim.x * blockDim.x;
    double2* U[3] = {a.u0, a.u1, a.u2};
    for (int32_t step = 0; step < a.n_steps; ++step) {
        const double F = a.Fn[step], Fp = a.Fo[step];
        double2* un = U[step % 3];          // u_n
        double2* um = U[(step + 2) % 3];    // u_{n-1}
        double2* ux = U[(step + 1) % 3];    // iterate, u_{n+1} at the end of the step
        const bool ext = a.extrapolate && step > 0;
        // phase R: b = (2M/k - A_re - Fp^2 M_D - i Fp E) u_n, r = b - A(F) x0 with
        // x0 = 2 u_n - u_{n-1} (or u_n)
        double red[kRedS] = {0.0, 0.0, 0.0, 0.0};
        sbc_spmv<true>(a, un, um, ext, -1.0, -Fp * Fp, 2.0 * a.inv_k, -Fp, 1.0, F * F, 0.0, F,
                       [&](int64_t i, double2 b, double2 ax) {
            const double2 ri = make_double2(b.x - ax.x, b.y - ax.y);
            const int32_t d = a.diag[i];
            a.dinv[i] = cinv(make_double2(a.are[d] + F * F * a.mdg[d], F * a.eg[d]));
            a.r[i] = ri;
            a.rh[i] = ri;
            a.p[i] = make_double2(0.0, 0.0);
            a.v[i] = make_double2(0.0, 0.0);
            const double2 uc = un[i];
            if (ext) {
                const double2 uo = um[i];
                ux[i] = make_double2(2.0 * uc.x - uo.x, 2.0 * uc.y - uo.y);
            } else {
                ux[i] = uc;
            }
            red[0] += b.x * b.x + b.y * b.y;
            red[1] += ri.x * ri.x + ri.y * ri.y;
        });
        if (!sbc_reduce(red, a, nb, flip, gen, sm)) return;
        const double bb = red[0];
        double rr = red[1];
        double2 rho = make_double2(rr, 0.0), rho_old = make_double2(1.0, 0.0);
        double2 alpha = make_double2(1.0, 0.0), omega = make_double2(1.0, 0.0);
        const double tol2 = a.rtol2 * bb;
        int it = 0;
        bool first = true;
        while (rr > tol2) {
            if (it >= a.maxit || (rho.x == 0.0 && rho.y == 0.0)) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
                return;
            }
            // p = r + beta (p - omega v),  beta = (rho / rho_old)(alpha / omega);  y = D^-1 p
            const double2 beta = first ? make_double2(0.0, 0.0) : cmul(cdiv(rho, rho_old), cdiv(alpha, omega));
            for (int64_t i = gt; i < a.n; i += nt) {
                const double2 pv = a.p[i], vv = a.v[i], rv = a.r[i];
                const double2 pw = make_double2(pv.x - (omega.x * vv.x - omega.y * vv.y),
                                                pv.y - (omega.x * vv.y + omega.y * vv.x));
                const double2 bp = cmul(beta, pw);
                const double2 pn = make_double2(rv.x + bp.x, rv.y + bp.y);
                a.p[i] = pn;
                a.y[i] = cmul(a.dinv[i], pn);
            }
            first = false;
            if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return;
            // v = A y ; (rh, v)
            double r2[kRedS] = {0.0, 0.0, 0.0, 0.0};
            sbc_apply(a, a.y, [&](int64_t i, double2 vi) {
                a.v[i] = vi;
                const double2 c = cdotc(a.rh[i], vi);
                r2[0] += c.x;
                r2[1] += c.y;
            });
            if (!sbc_reduce(r2, a, nb, flip, gen, sm)) return;
            const double2 rv = make_double2(r2[0], r2[1]);
            if (rv.x == 0.0 && rv.y == 0.0) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
                return;
            }
            alpha = cdiv(rho, rv);
            // s = r - alpha v ; z = D^-1 s
            for (int64_t i = gt; i < a.n; i += nt) {
                const double2 av = cmul(alpha, a.v[i]);
                const double2 rv2 = a.r[i];
                const double2 si = make_double2(rv2.x - av.x, rv2.y - av.y);
                a.sv[i] = si;
                a.z[i] = cmul(a.dinv[i], si);
            }
            if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return;
            // t = A z ; (t, s), (t, t), (s, s)
            double r4[kRedS] = {0.0, 0.0, 0.0, 0.0};
            sbc_apply(a, a.z, [&](int64_t i, double2 ti) {
                a.t[i] = ti;
                const double2 si = a.sv[i];
                const double2 c = cdotc(ti, si);
                r4[0] += c.x;
                r4[1] += c.y;
                r4[2] += ti.x * ti.x + ti.y * ti.y;
                r4[3] += si.x * si.x + si.y * si.y;
            });
            if (!sbc_reduce(r4, a, nb, flip, gen, sm)) return;
            ++it;
            if (r4[3] <= tol2 || r4[2] == 0.0) {
                // s is already small enough (or t vanished): x += alpha y, r = s
                for (int64_t i = gt; i < a.n; i += nt) {
                    const double2 ay = cmul(alpha, a.y[i]);
                    const double2 xv = ux[i];
                    ux[i] = make_double2(xv.x + ay.x, xv.y + ay.y);
                    a.r[i] = a.sv[i];
                }
                rr = r4[3];
                break;
            }
            omega = make_double2(r4[0] / r4[2], r4[1] / r4[2]);
            // x += alpha y + omega z ; r = s - omega t ; (rh, r), (r, r)
            double r3[kRedS] = {0.0, 0.0, 0.0, 0.0};
            for (int64_t i = gt; i < a.n; i += nt) {
                const double2 ay = cmul(alpha, a.y[i]), oz = cmul(omega, a.z[i]), ot = cmul(omega, a.t[i]);
                const double2 xv = ux[i], si = a.sv[i];
                ux[i] = make_double2(xv.x + ay.x + oz.x, xv.y + ay.y + oz.y);
                const double2 rn = make_double2(si.x - ot.x, si.y - ot.y);
                a.r[i] = rn;
                const double2 c = cdotc(a.rh[i], rn);
                r3[0] += c.x;
                r3[1] += c.y;
                r3[2] += rn.x * rn.x + rn.y * rn.y;
            }
            if (!sbc_reduce(r3, a, nb, flip, gen, sm)) return;
            rho_old = rho;
            rho = make_double2(r3[0], r3[1]);
            rr = r3[2];
            if (omega.x == 0.0 && omega.y == 0.0) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
                return;
            }
        }
        if (gt == 0) {
            a.iters[step] = it;
            a.relres[step] = bb > 0.0 ? sqrt(rr / bb) : 0.0;
        }
        // the next phase R gathers u_n, u_{n-1} and writes the third buffer
        if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return;
    }
    // signal: sum_i w_i Re(u_i), total and per compartment
    const double2* uN = U[a.n_steps % 3];
    double sg[kRedS] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = gt; i < a.n; i += nt) {
        const double c = a.w[i] * uN[i].x;
        sg[0] += c;
        const int rc = a.rcomp[i];
        if (rc == 0) sg[1] += c;
        else if (rc == 1) sg[2] += c;
    }
    if (!sbc_reduce(sg, a, nb, flip, gen, sm)) return;
    if (gt == 0) {
        a.out[0] = sg[0];
        a.out[1] = sg[1];
        a.out[2] = sg[2];
    }
}

// ----------------------------------------------------- batched stepper --
// Up to 32 signals of one sequence in one cooperative launch: a warp takes a
// row, its lane l the row's value of signal l, so each stored entry (column,
// M/k + theta S, the six M_D and three E components) is read once for all of
// them; lane l forms its signal's (M_D)_g and E_g from its own direction and
// scales them by theta q^2 F^2 and theta q F.  Every signal runs its
// own Jacobi-BiCGSTAB (its own rho, alpha, omega; a converged signal stops
// moving) and the launch iterates until all have converged.  Sums over rows go
// per signal through two-stage grid reductions (block partials; one warp per
// value over the blocks; the results read by every block), fixed order.
constexpr int kMR = 32;   // signals per batched launch (lanes)
constexpr int kMV = 4;    // values per signal in one reduction

struct SbcMultiArgs {
    int64_t n;
    const int32_t* __restrict__ row_ptr;
    const int32_t* __restrict__ col;
    const int32_t* __restrict__ diag;
    const int32_t* __restrict__ rcomp;
    const double* __restrict__ m;
    const double* __restrict__ are;
    const double* __restrict__ md6;  // six M_D components per entry (xx, yy, zz, 2xy, 2xz, 2yz)
    const double* __restrict__ e3;   // three E components per entry (g_x, g_y, g_z)
    const double* __restrict__ md;   // one direction for all lanes (nullable): theta (M_D)_g per entry
    const double* __restrict__ ev;   //   and theta E_g per entry
    const double* __restrict__ w;
    const double* __restrict__ q;    // [kMR]
    const double* __restrict__ gl;   // [kMR][3] unit gradient direction per signal
    double theta;
    const double* __restrict__ Fn;   // [kMR][n_steps]
    const double* __restrict__ Fo;
    double inv_k;
    int32_t R, n_steps, maxit, extrapolate;
    double rtol2;
    double2 *u0, *u1, *u2, *r, *rh, *p, *v, *sv, *t, *y, *z, *dinv;   // [n][kMR]
    double* partials;                // [2][nb][kMR * kMV]
    double* fin;                     // [kMR * kMV]
    unsigned* bar;
    int* status;
    int32_t* iters;                  // [n_steps]
    double* relres;                  // [kMR][n_steps]
    double* out;                     // [kMR][3]
    unsigned long long wait_ns;
};

// Per-signal sums: v[k] of this lane (its signal) summed over every row-warp of
// the grid; on return v holds the totals (every lane of every block).
__device__ __forceinline__ bool sbcm_reduce(double (&v)[kMV], const SbcMultiArgs& a, unsigned nb, unsigned& flip,
                                            unsigned& gen, double* sm /* [kWarps * kMR * kMV] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    constexpr int V = kMR * kMV;
#pragma unroll
    for (int k = 0; k < kMV; ++k) sm[(wid * kMR + lane) * kMV + k] = v[k];
    __syncthreads();
    double* P = a.partials + (size_t)(flip & 1u) * nb * V;
    ++flip;
    for (int t = threadIdx.x; t < V; t += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += sm[w * V + t];
        P[(size_t)blockIdx.x * V + t] = s;
    }
    if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return false;
    // stage 2: warp gw of the grid sums value gw over the blocks
    const unsigned gw = blockIdx.x * nw + wid;
    for (unsigned t = gw; t < (unsigned)V; t += nb * nw) {
        double s = 0.0;
        for (unsigned b = lane; b < nb; b += 32) s += __ldcg(&P[(size_t)b * V + t]);
        s = warp_sum(s);
        if (lane == 0) a.fin[t] = s;
    }
    if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return false;
#pragma unroll
    for (int k = 0; k < kMV; ++k) v[k] = __ldcg(&a.fin[lane * kMV + k]);
    __syncthreads();
    return true;
}

__global__ void __launch_bounds__(kThreadsS, 1) k_step_sbc_multi(SbcMultiArgs a) {
    __shared__ double sm[(kThreadsS / 32) * kMR * kMV];
    const unsigned nb = gridDim.x;
    unsigned gen = 0, flip = 0;
    const int lane = threadIdx.x & 31;
    const bool live = lane < a.R;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const double ql = live ? a.q[lane] : 0.0;
    const double gx = live ? a.gl[lane * 3] : 0.0, gy = live ? a.gl[lane * 3 + 1] : 0.0,
                 gz = live ? a.gl[lane * 3 + 2] : 0.0;
    const double gg[6] = {gx * gx, gy * gy, gz * gz, gx * gy, gx * gz, gy * gz};
    // this signal's theta (M_D)_g and theta E_g of stored entry e
    // (a group of one direction reads them precombined)
    const bool shared = a.md != nullptr;
    auto mdg = [&](int32_t e) {
        if (shared) return a.md[e];
        const double* d = a.md6 + (size_t)6 * e;
        return a.theta * (d[0] * gg[0] + d[1] * gg[1] + d[2] * gg[2] + d[3] * gg[3] + d[4] * gg[4] + d[5] * gg[5]);
    };
    auto eg = [&](int32_t e) {
        if (shared) return a.ev[e];
        const double* d = a.e3 + (size_t)3 * e;
        return a.theta * (d[0] * gx + d[1] * gy + d[2] * gz);
    };
    double2* U[3] = {a.u0, a.u1, a.u2};
    for (int32_t step = 0; step < a.n_steps; ++step) {
        const double F = live ? a.Fn[(size_t)lane * a.n_steps + step] : 0.0;
        const double Fp = live ? a.Fo[(size_t)lane * a.n_steps + step] : 0.0;
        const double c2 = ql * ql * F * F, c1 = ql * F, p2 = ql * ql * Fp * Fp, p1 = ql * Fp;
        double2* un = U[step % 3];
        double2* um = U[(step + 2) % 3];
        double2* ux = U[(step + 1) % 3];
        const bool ext = a.extrapolate && step > 0;
        // phase R: b = (2M/k - A_re - Fp^2 q^2 M_D - i Fp q E) u_n, x0 = 2 u_n - u_{n-1},
        // r = b - A(F) x0, Jacobi inverse
        double red[kMV] = {0.0, 0.0, 0.0, 0.0};
        for (int64_t row = gw; row < a.n; row += nwarps) {
            const size_t vi = (size_t)row * kMR + lane;
            double2 b = make_double2(0.0, 0.0), ax = make_double2(0.0, 0.0);
            const int32_t e0 = a.row_ptr[row], e1 = a.row_ptr[row + 1];
            for (int32_t e = e0; e < e1; ++e) {
                const size_t cj = (size_t)a.col[e] * kMR + lane;
                const double ar = a.are[e], mdv = mdg(e), mm = a.m[e], evv = eg(e);
                const double2 xv = un[cj];
                double2 x0 = xv;
                if (ext) {
                    const double2 xo = um[cj];
                    x0 = make_double2(2.0 * xv.x - xo.x, 2.0 * xv.y - xo.y);
                }
                const double rb = 2.0 * a.inv_k * mm - ar - p2 * mdv, ib = -p1 * evv;
                b.x += rb * xv.x - ib * xv.y;
                b.y += rb * xv.y + ib * xv.x;
                const double ra = ar + c2 * mdv, ia = c1 * evv;
                ax.x += ra * x0.x - ia * x0.y;
                ax.y += ra * x0.y + ia * x0.x;
            }
            const int32_t d = a.diag[row];
            const double2 ri = make_double2(b.x - ax.x, b.y - ax.y);
            a.dinv[vi] = cinv(make_double2(a.are[d] + c2 * mdg(d), c1 * eg(d)));
            a.r[vi] = ri;
            a.rh[vi] = ri;
            a.p[vi] = make_double2(0.0, 0.0);
            a.v[vi] = make_double2(0.0, 0.0);
            const double2 uc = un[vi];
            if (ext) {
                const double2 uo = um[vi];
                ux[vi] = make_double2(2.0 * uc.x - uo.x, 2.0 * uc.y - uo.y);
            } else {
                ux[vi] = uc;
            }
            red[0] += b.x * b.x + b.y * b.y;
            red[1] += ri.x * ri.x + ri.y * ri.y;
        }
        if (!sbcm_reduce(red, a, nb, flip, gen, sm)) return;
        const double bb = red[0], tol2 = a.rtol2 * red[0];
        double rr = red[1];
        bool act = live && rr > tol2;
        double2 rho = make_double2(rr, 0.0), rho_old = make_double2(1.0, 0.0);
        double2 alpha = make_double2(1.0, 0.0), omega = make_double2(1.0, 0.0);
        bool first = true;
        int it = 0;
        while (__syncthreads_or(act)) {   // the same in every block: the sums are grid-identical
            if (it >= a.maxit) {
                if (threadIdx.x == 0) atomicCAS(a.status, DEV_OK, DEV_NOT_CONVERGED);
                return;
            }
            if (act && rho.x == 0.0 && rho.y == 0.0) {
                atomicCAS(a.status, DEV_OK, DEV_BREAKDOWN);
                act = false;
            }
            // p = r + beta (p - omega v), y = D^-1 p
            const double2 beta = first ? make_double2(0.0, 0.0) : cmul(cdiv(rho, rho_old), cdiv(alpha, omega));
            first = false;
            if (act)
                for (int64_t row = gw; row < a.n; row += nwarps) {
                    const size_t vi = (size_t)row * kMR + lane;
                    const double2 pv = a.p[vi], vv = a.v[vi], rv = a.r[vi];
                    const double2 pw = make_double2(pv.x - (omega.x * vv.x - omega.y * vv.y),
                                                    pv.y - (omega.x * vv.y + omega.y * vv.x));
                    const double2 bp = cmul(beta, pw);
                    const double2 pn = make_double2(rv.x + bp.x, rv.y + bp.y);
                    a.p[vi] = pn;
                    a.y[vi] = cmul(a.dinv[vi], pn);
                }
            if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return;
            // v = A y ; (rh, v)
            double r2[kMV] = {0.0, 0.0, 0.0, 0.0};
            if (act)
                for (int64_t row = gw; row < a.n; row += nwarps) {
                    const size_t vi = (size_t)row * kMR + lane;
                    double2 acc = make_double2(0.0, 0.0);
                    for (int32_t e = a.row_ptr[row]; e < a.row_ptr[row + 1]; ++e) {
                        const double ra = a.are[e] + c2 * mdg(e), ia = c1 * eg(e);
                        const double2 xv = a.y[(size_t)a.col[e] * kMR + lane];
                        acc.x += ra * xv.x - ia * xv.y;
                        acc.y += ra * xv.y + ia * xv.x;
                    }
                    a.v[vi] = acc;
                    const double2 c = cdotc(a.rh[vi], acc);
                    r2[0] += c.x;
                    r2[1] += c.y;
                }
            if (!sbcm_reduce(r2, a, nb, flip, gen, sm)) return;
            const double2 rv = make_double2(r2[0], r2[1]);
            if (act && rv.x == 0.0 && rv.y == 0.0) {
                atomicCAS(a.status, DEV_OK, DEV_BREAKDOWN);
                act = false;
            }
            if (act) alpha = cdiv(rho, rv);
            // s = r - alpha v ; z = D^-1 s
            if (act)
                for (int64_t row = gw; row < a.n; row += nwarps) {
                    const size_t vi = (size_t)row * kMR + lane;
                    const double2 av = cmul(alpha, a.v[vi]), rv2 = a.r[vi];
                    const double2 si = make_double2(rv2.x - av.x, rv2.y - av.y);
                    a.sv[vi] = si;
                    a.z[vi] = cmul(a.dinv[vi], si);
                }
            if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return;
            // t = A z ; (t, s), (t, t), (s, s)
            double r4[kMV] = {0.0, 0.0, 0.0, 0.0};
            if (act)
                for (int64_t row = gw; row < a.n; row += nwarps) {
                    const size_t vi = (size_t)row * kMR + lane;
                    double2 acc = make_double2(0.0, 0.0);
                    for (int32_t e = a.row_ptr[row]; e < a.row_ptr[row + 1]; ++e) {
                        const double ra = a.are[e] + c2 * mdg(e), ia = c1 * eg(e);
                        const double2 xv = a.z[(size_t)a.col[e] * kMR + lane];
                        acc.x += ra * xv.x - ia * xv.y;
                        acc.y += ra * xv.y + ia * xv.x;
                    }
                    a.t[vi] = acc;
                    const double2 si = a.sv[vi];
                    const double2 c = cdotc(acc, si);
                    r4[0] += c.x;
                    r4[1] += c.y;
                    r4[2] += acc.x * acc.x + acc.y * acc.y;
                    r4[3] += si.x * si.x + si.y * si.y;
                }
            if (!sbcm_reduce(r4, a, nb, flip, gen, sm)) return;
            ++it;
            // this signal's s is already small enough (or t vanished): x += alpha y, r = s, done
            const bool early = act && (r4[3] <= tol2 || r4[2] == 0.0);
            if (act) omega = early ? make_double2(0.0, 0.0) : make_double2(r4[0] / r4[2], r4[1] / r4[2]);
            // x += alpha y + omega z ; r = s - omega t ; (rh, r), (r, r)
            double r3[kMV] = {0.0, 0.0, 0.0, 0.0};
            if (act)
                for (int64_t row = gw; row < a.n; row += nwarps) {
                    const size_t vi = (size_t)row * kMR + lane;
                    const double2 ay = cmul(alpha, a.y[vi]), oz = cmul(omega, a.z[vi]), ot = cmul(omega, a.t[vi]);
                    const double2 xv = ux[vi], si = a.sv[vi];
                    ux[vi] = make_double2(xv.x + ay.x + oz.x, xv.y + ay.y + oz.y);
                    const double2 rn = make_double2(si.x - ot.x, si.y - ot.y);
                    a.r[vi] = rn;
                    const double2 c = cdotc(a.rh[vi], rn);
                    r3[0] += c.x;
                    r3[1] += c.y;
                    r3[2] += rn.x * rn.x + rn.y * rn.y;
                }
            if (!sbcm_reduce(r3, a, nb, flip, gen, sm)) return;
            if (act) {
                rho_old = rho;
                rho = make_double2(r3[0], r3[1]);
                rr = r3[2];
                if (early || rr <= tol2) act = false;
                else if (omega.x == 0.0 && omega.y == 0.0) {
                    atomicCAS(a.status, DEV_OK, DEV_BREAKDOWN);
                    act = false;
                }
            }
        }
        if (blockIdx.x == 0 && threadIdx.x < 32) {
            if (threadIdx.x == 0) a.iters[step] = it;
            if (live) a.relres[(size_t)lane * a.n_steps + step] = bb > 0.0 ? sqrt(rr / bb) : 0.0;
        }
        if (!grid_barrier(a.bar, nb, a.status, gen, a.wait_ns)) return;
    }
    // signals: sum_i w_i Re(u_i), total and per compartment
    const double2* uN = U[a.n_steps % 3];
    double sg[kMV] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t row = gw; row < a.n; row += nwarps) {
        const double c = a.w[row] * uN[(size_t)row * kMR + lane].x;
        sg[0] += c;
        const int rc = a.rcomp[row];
        if (rc == 0) sg[1] += c;
        else if (rc == 1) sg[2] += c;
    }
    if (!sbcm_reduce(sg, a, nb, flip, gen, sm)) return;
    if (blockIdx.x == 0 && threadIdx.x < 32 && live) {
        a.out[lane * 3 + 0] = sg[0];
        a.out[lane * 3 + 1] = sg[1];
        a.out[lane * 3 + 2] = sg[2];
    }
}

// Initial state of every lane of the batched stepper, and the lane -> signal
// copy of the final states.
__global__ void k_sbcm_init(int64_t n, const int32_t* __restrict__ u0_vertex, const double* __restrict__ u0,
                            double2* __restrict__ u) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * kMR; i += (int64_t)gridDim.x * blockDim.x)
        u[i] = make_double2(u0 ? u0[u0_vertex[i / kMR]] : 1.0, 0.0);
}

__global__ void k_sbcm_extract(int64_t n, int lane, const double2* __restrict__ u, double2* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = u[i * kMR + lane];
}

// ------------------------------------------------------------------ host --
static void map_status_sbc(int st) {
    switch (st) {
        case DEV_OK: return;
        case DEV_TIMEOUT: throw Error(BT_ERR_TIMEOUT, "strong periodic stepper: a grid-wide wait ran out");
        case DEV_NOT_CONVERGED:
            throw Error(BT_ERR_NOT_CONVERGED, "strong periodic stepper: BiCGSTAB reached max_iterations or broke down");
        case DEV_BREAKDOWN: throw Error(BT_ERR_BREAKDOWN, "strong periodic stepper: BiCGSTAB breakdown");
        default: throw Error(BT_ERR_CUDA, "strong periodic stepper: device error");
    }
}

void set_strong(bt_ctx* ctx, const int32_t* dir) {
    if (!ctx->strong) ctx->strong = new Strong();
    Strong& P = *ctx->strong;
    for (int d = 0; d < 3; ++d) {
        BT_REQUIRE(dir[d] == 0 || dir[d] == 1, BT_ERR_INVALID, "periodic directions must be 0 or 1");
        P.dir[d] = dir[d];
    }
    P.on = dir[0] || dir[1] || dir[2];
    P.built_version = -1;
}

bool strong_active(const bt_ctx* ctx) { return ctx->strong && ctx->strong->on; }

// One launch of the batched stepper for the signals grp (one sequence, 3..32
// signals, any directions); outputs go to the signals' places in the call.
static float run_strong_multi(bt_ctx* ctx, Strong& P, const std::vector<int32_t>& grp, const double* q,
                              const double* gdir, const int32_t* seq, const double* d_u0, double rtol, int32_t maxit,
                              double* sig, double* comp_sig, bt_stats* st) {
    Schedule& S = ctx->sched;
    Mesh& m = ctx->mesh;
    cudaStream_t s = ctx->stream;
    const int64_t n = P.n, nnz = P.nnz;
    const int R = (int)grp.size();
    int per_sm = 0;
    BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_sbc_multi, kThreadsS, 0));
    BT_REQUIRE(per_sm >= 1, BT_ERR_CUDA, "strong periodic batched stepper does not fit on an SM");
    const int64_t need = std::max<int64_t>(1, (n + kThreadsS / 32 - 1) / (kThreadsS / 32));   // a warp per row
    P.mblocks = (int32_t)std::min<int64_t>((int64_t)per_sm * ctx->num_sms, need);
    const size_t vn = (size_t)n * kMR;
    for (auto* b : {&P.mu[0], &P.mu[1], &P.mu[2], &P.mr, &P.mrh, &P.mp, &P.mv, &P.ms, &P.mt, &P.my, &P.mz, &P.mdinv}) {
        b->alloc(vn);
        b->zero(s);
    }
    P.mpart.alloc((size_t)2 * P.mblocks * kMR * kMV);
    P.mfin.alloc((size_t)kMR * kMV);
    P.mout.alloc((size_t)kMR * 3);
    P.mrel.alloc((size_t)kMR * S.n_steps);
    P.iters.alloc(S.n_steps);
    P.bar.alloc(4);
    P.status.alloc(1);
    // are = M/k + theta S; when every signal of the group has one direction, also
    // that direction's theta (M_D)_g and theta E_g (unit q), else each lane forms its own
    bool one_dir = true;
    const double* g0 = gdir + 3 * grp.front();
    const double g0n = std::sqrt(g0[0] * g0[0] + g0[1] * g0[1] + g0[2] * g0[2]);
    for (int l = 1; l < R; ++l) {
        const double* g = gdir + 3 * grp[l];
        const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        for (int k = 0; k < 3; ++k) one_dir = one_dir && g[k] / gn == g0[k] / g0n;
    }
    P.are.alloc(nnz);
    P.mdg.alloc(nnz);
    P.eg.alloc(nnz);
    const int pack_blocks = (int)std::min<int64_t>((nnz + 255) / 256, (int64_t)ctx->num_sms * 8);
    k_sbc_pack<<<std::max(1, pack_blocks), 256, 0, s>>>(nnz, P.m, P.s, P.md6, P.e3, 1.0 / S.dt, S.theta, 1.0,
                                                         g0[0] / g0n, g0[1] / g0n, g0[2] / g0n, P.are, P.mdg, P.eg);
    BT_CUDA(cudaGetLastError());
    std::vector<double> hq(kMR, 0.0), hg((size_t)kMR * 3, 0.0), hFn((size_t)kMR * S.n_steps, 0.0),
        hFo((size_t)kMR * S.n_steps, 0.0);
    const int32_t srow = seq ? seq[grp.front()] : 0;
    BT_REQUIRE(srow >= 0 && srow < S.n_seq, BT_ERR_INVALID, "sequence index out of range");
    for (int l = 0; l < R; ++l) {
        hq[l] = q[grp[l]];
        const double* g = gdir + 3 * grp[l];
        const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        for (int k = 0; k < 3; ++k) hg[(size_t)l * 3 + k] = g[k] / gn;
        for (int k = 0; k < S.n_steps; ++k) {
            hFn[(size_t)l * S.n_steps + k] = S.F_new[(size_t)srow * S.n_steps + k];
            hFo[(size_t)l * S.n_steps + k] = S.F_old[(size_t)srow * S.n_steps + k];
        }
    }
    P.mq.upload(hq.data(), kMR, s);
    P.mg.upload(hg.data(), hg.size(), s);
    P.mFn.upload(hFn.data(), hFn.size(), s);
    P.mFo.upload(hFo.data(), hFo.size(), s);
    const int init_blocks = (int)std::min<int64_t>((int64_t)((vn + 255) / 256), (int64_t)ctx->num_sms * 8);
    k_sbcm_init<<<std::max(1, init_blocks), 256, 0, s>>>(n, P.u0_vertex, d_u0, P.mu[0]);
    BT_CUDA(cudaGetLastError());
    P.bar.zero(s);
    P.status.zero(s);
    SbcMultiArgs a{};
    a.n = n;
    a.row_ptr = P.row_ptr;
    a.col = P.col;
    a.diag = P.diag;
    a.rcomp = P.rcomp;
    a.m = P.m;
    a.are = P.are;
    a.md6 = P.md6;
    a.e3 = P.e3;
    a.md = one_dir ? P.mdg.p : nullptr;
    a.ev = one_dir ? P.eg.p : nullptr;
    a.gl = P.mg;
    a.theta = S.theta;
    a.w = P.w;
    a.q = P.mq;
    a.Fn = P.mFn;
    a.Fo = P.mFo;
    a.inv_k = 1.0 / S.dt;
    a.R = R;
    a.n_steps = S.n_steps;
    a.maxit = maxit;
    a.extrapolate = ctx->opt_fp64_extrapolate >= 1 ? 1 : 0;
    a.rtol2 = rtol * rtol;
    a.u0 = P.mu[0];
    a.u1 = P.mu[1];
    a.u2 = P.mu[2];
    a.r = P.mr;
    a.rh = P.mrh;
    a.p = P.mp;
    a.v = P.mv;
    a.sv = P.ms;
    a.t = P.mt;
    a.y = P.my;
    a.z = P.mz;
    a.dinv = P.mdinv;
    a.partials = P.mpart;
    a.fin = P.mfin;
    a.bar = P.bar;
    a.status = P.status;
    a.iters = P.iters;
    a.relres = P.mrel;
    a.out = P.mout;
    a.wait_ns = ctx->opt_wait_ns;
    void* args[] = {&a};
    BT_CUDA(cudaEventRecord(ctx->ev1, s));
    BT_CUDA(cudaLaunchCooperativeKernel((const void*)k_step_sbc_multi, dim3(P.mblocks), dim3(kThreadsS), args, 0, s));
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    int hst = 0;
    std::vector<double> hout((size_t)kMR * 3), hrel((size_t)kMR * S.n_steps);
    std::vector<int32_t> hit(S.n_steps);
    P.status.download(&hst, 1, s);
    P.mout.download(hout.data(), hout.size(), s);
    P.mrel.download(hrel.data(), hrel.size(), s);
    P.iters.download(hit.data(), S.n_steps, s);
    BT_CUDA(cudaStreamSynchronize(s));
    map_status_sbc(hst);
    float ms = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2));
    const unsigned eb = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8);
    for (int l = 0; l < R; ++l) {
        const int32_t sg = grp[l];
        k_sbcm_extract<<<std::max(1u, eb), 256, 0, s>>>(n, l, P.mu[S.n_steps % 3], P.saved.p + (size_t)sg * n);
        sig[sg] = hout[(size_t)l * 3];
        if (comp_sig)
            for (int c = 0; c < m.n_comp && c < 2; ++c) comp_sig[(size_t)sg * m.n_comp + c] = hout[(size_t)l * 3 + 1 + c];
        for (int k = 0; k < S.n_steps; ++k) {
            ctx->last_iters[(size_t)sg * S.n_steps + k] = hit[k];
            if (st) {
                st->max_iterations = std::max(st->max_iterations, hit[k]);
                st->total_iterations += hit[k];
                st->max_rel_residual = std::max(st->max_rel_residual, hrel[(size_t)l * S.n_steps + k]);
            }
        }
    }
    BT_CUDA(cudaGetLastError());
    if (st) st->kernel_launches += 3 + R;
    return ms;
}

void solve_strong(bt_ctx* ctx, int32_t nsig, const double* q, const double* gdir, const int32_t* seq,
                  const double* u0, double rtol, int32_t maxit, double* sig, double* comp_sig, bt_stats* st) {
    Strong& P = *ctx->strong;
    Schedule& S = ctx->sched;
    Mesh& m = ctx->mesh;
    cudaStream_t s = ctx->stream;
    BT_REQUIRE(S.F_new.size() == (size_t)S.n_steps * S.n_seq && S.F_old.size() == (size_t)S.n_steps * S.n_seq,
               BT_ERR_STATE, "strong pseudo-periodic form needs bt_set_schedule_integral (F at both levels)");
    if (P.built_version != ctx->mat.version) {
        build_strong(ctx, P);
        P.built_version = ctx->mat.version;
    }
    for (int32_t sg = 0; sg < nsig; ++sg) {
        const double* g = gdir + 3 * sg;
        const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        BT_REQUIRE(gn > 0.0, BT_ERR_INVALID, "gradient direction must be non-zero");
        for (int k = 0; k < 3; ++k)
            BT_REQUIRE(!(P.excess_dir[k] && std::fabs(g[k] / gn) > 1e-12), BT_ERR_INVALID,
                       "strong periodic form: (D g).n must vanish on exterior facets off the periodic faces that "
                       "touch a compartment interface (the reference's phase-blind outer term acts there)");
    }
    const int64_t n = P.n, nnz = P.nnz;
    int per_sm = 0;
    BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_sbc, kThreadsS, 0));
    BT_REQUIRE(per_sm >= 1, BT_ERR_CUDA, "strong periodic stepper does not fit on an SM");
    // one thread per row at least, and (small systems) one block per SM with >= 16
    // rows each: the stepper is bound by FP64 latency, so it spreads over the SMs
    const int64_t need = std::max<int64_t>((n + kThreadsS - 1) / kThreadsS,
                                           std::min<int64_t>(ctx->num_sms, (n + 15) / 16));
    P.nblocks = (int32_t)std::max<int64_t>(1, std::min<int64_t>((int64_t)per_sm * ctx->num_sms, need));
    P.are.alloc(nnz);
    P.mdg.alloc(nnz);
    P.eg.alloc(nnz);
    for (auto* b : {&P.u[0], &P.u[1], &P.u[2], &P.r, &P.rh, &P.p, &P.v, &P.sv, &P.t, &P.y, &P.z, &P.dinv})
        b->alloc(n);
    P.ac.alloc(nnz);
    P.partials.alloc((size_t)2 * P.nblocks * kRedS);
    P.out.alloc(kRedS);
    P.relres.alloc(S.n_steps);
    P.iters.alloc(S.n_steps);
    P.bar.alloc(4);
    P.status.alloc(1);
    P.saved.alloc((size_t)nsig * n);
    P.saved_nsig = nsig;
    DevBuf<double> d_u0;
    if (u0) d_u0.upload(u0, m.n_v, s);
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
    std::vector<double> hFn(S.n_steps), hFo(S.n_steps), hres(S.n_steps), hout(kRedS);
    std::vector<int32_t> hit(S.n_steps);
    float stepper_ms = 0.0f;
    // signals of one sequence go through the batched stepper in groups of up to 32
    // (any directions); a group of one or two takes the single-signal stepper
    std::vector<std::vector<int32_t>> groups;
    {
        std::vector<int32_t> ord(nsig);
        for (int32_t i = 0; i < nsig; ++i) ord[i] = i;
        auto key = [&](int32_t i) { return seq ? seq[i] : 0; };
        // by sequence, then direction: a b-series of one direction fills a launch
        // that reads its direction terms precombined
        auto dir = [&](int32_t i) {
            const double* g = gdir + 3 * i;
            const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            return std::array<double, 3>{g[0] / gn, g[1] / gn, g[2] / gn};
        };
        std::stable_sort(ord.begin(), ord.end(), [&](int32_t x, int32_t y) {
            if (key(x) != key(y)) return key(x) < key(y);
            return dir(x) < dir(y);
        });
        for (int32_t i = 0; i < nsig; ++i) {
            if (ctx->opt_strong_batch && !groups.empty() && key(groups.back().front()) == key(ord[i]) &&
                (int)groups.back().size() < kMR)
                groups.back().push_back(ord[i]);
            else
                groups.push_back({ord[i]});
        }
    }
    BT_CUDA(cudaEventRecord(ctx->ev0, s));
    // (a batched launch costs about what one single-signal launch does on small
    // systems, so it pays from three signals on)
    for (const auto& grp : groups) {
      if (grp.size() >= 3) {
        stepper_ms += run_strong_multi(ctx, P, grp, q, gdir, seq, u0 ? d_u0.p : nullptr, rtol, maxit, sig, comp_sig, st);
        continue;
      }
      for (const int32_t sg : grp) {
        const int32_t row = seq ? seq[sg] : 0;
        BT_REQUIRE(row >= 0 && row < S.n_seq, BT_ERR_INVALID, "sequence index out of range");
        for (int k = 0; k < S.n_steps; ++k) {
            hFn[k] = S.F_new[(size_t)row * S.n_steps + k];
            hFo[k] = S.F_old[(size_t)row * S.n_steps + k];
        }
        P.Fn.upload(hFn.data(), S.n_steps, s);
        P.Fo.upload(hFo.data(), S.n_steps, s);
        const double* g = gdir + 3 * sg;
        const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        const int pack_blocks = (int)std::min<int64_t>((nnz + 255) / 256, (int64_t)ctx->num_sms * 8);
        k_sbc_pack<<<std::max(1, pack_blocks), 256, 0, s>>>(nnz, P.m, P.s, P.md6, P.e3, 1.0 / S.dt, S.theta, q[sg],
                                                             g[0] / gn, g[1] / gn, g[2] / gn, P.are, P.mdg, P.eg);
        BT_CUDA(cudaGetLastError());
        const int init_blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8);
        k_sbc_init<<<std::max(1, init_blocks), 256, 0, s>>>(n, P.u0_vertex, u0 ? d_u0.p : nullptr, P.u[0]);
        BT_CUDA(cudaGetLastError());
        P.bar.zero(s);
        P.status.zero(s);
        SbcArgs a{};
        a.n = n;
        a.row_ptr = P.row_ptr;
        a.col = P.col;
        a.diag = P.diag;
        a.rcomp = P.rcomp;
        a.m = P.m;
        a.are = P.are;
        a.mdg = P.mdg;
        a.eg = P.eg;
        a.w = P.w;
        a.Fn = P.Fn;
        a.Fo = P.Fo;
        a.inv_k = 1.0 / S.dt;
        a.u0 = P.u[0];
        a.u1 = P.u[1];
        a.u2 = P.u[2];
        a.extrapolate = ctx->opt_fp64_extrapolate >= 1 ? 1 : 0;
        a.r = P.r;
        a.rh = P.rh;
        a.p = P.p;
        a.v = P.v;
        a.sv = P.sv;
        a.t = P.t;
        a.y = P.y;
        a.z = P.z;
        a.dinv = P.dinv;
        a.ac = P.ac;
        a.partials = P.partials;
        a.bar = P.bar;
        a.status = P.status;
        a.iters = P.iters;
        a.relres = P.relres;
        a.out = P.out;
        a.n_steps = S.n_steps;
        a.maxit = maxit;
        a.nc = (int32_t)m.n_comp;
        a.rtol2 = rtol * rtol;
        a.wait_ns = ctx->opt_wait_ns;
        void* args[] = {&a};
        BT_CUDA(cudaEventRecord(ctx->ev1, s));
        BT_CUDA(cudaLaunchCooperativeKernel((const void*)k_step_sbc, dim3(P.nblocks), dim3(kThreadsS), args, 0, s));
        BT_CUDA(cudaEventRecord(ctx->ev2, s));
        int hst = 0;
        P.status.download(&hst, 1, s);
        P.out.download(hout.data(), kRedS, s);
        P.iters.download(hit.data(), S.n_steps, s);
        P.relres.download(hres.data(), S.n_steps, s);
        BT_CUDA(cudaStreamSynchronize(s));
        map_status_sbc(hst);
        float ms = 0.0f;
        BT_CUDA(cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2));
        stepper_ms += ms;
        BT_CUDA(cudaMemcpyAsync(P.saved.p + (size_t)sg * n, P.u[S.n_steps % 3].p, n * sizeof(double2),
                                cudaMemcpyDeviceToDevice, s));
        sig[sg] = hout[0];
        if (comp_sig)
            for (int c = 0; c < m.n_comp; ++c) comp_sig[(size_t)sg * m.n_comp + c] = hout[1 + c];
        for (int k = 0; k < S.n_steps; ++k) {
            ctx->last_iters[(size_t)sg * S.n_steps + k] = hit[k];
            if (st) {
                st->max_iterations = std::max(st->max_iterations, hit[k]);
                st->total_iterations += hit[k];
                st->max_rel_residual = std::max(st->max_rel_residual, hres[k]);
            }
        }
        if (st) st->kernel_launches += 3;
      }
    }
    BT_CUDA(cudaEventRecord(ctx->ev2, s));
    BT_CUDA(cudaEventSynchronize(ctx->ev2));
    float total_ms = 0.0f;
    BT_CUDA(cudaEventElapsedTime(&total_ms, ctx->ev0, ctx->ev2));
    if (st) {
        st->gpu_ms = total_ms;
        st->stepper_ms = stepper_ms;
    }
    ctx->last_nsig = nsig;
}

// Solution of signal `index` on the unfolded dofs (a slave dof takes its
// master's value).
void get_solution_strong(bt_ctx* ctx, int32_t index, double* u) {
    BT_REQUIRE(ctx->strong && index >= 0 && index < ctx->strong->saved_nsig, BT_ERR_INVALID,
               "bt_get_solution: no such signal in the last strong-periodic solve");
    Strong& P = *ctx->strong;
    std::vector<double2> h((size_t)P.n);
    P.saved.download(h.data(), P.n, ctx->stream);
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < P.fold.size(); ++i) {
        u[2 * i] = h[P.fold[i]].x;
        u[2 * i + 1] = h[P.fold[i]].y;
    }
}

void strong_info(const bt_ctx* ctx, int64_t* n_dofs, int64_t* nnz, int64_t* n_classes) {
    const Strong* P = ctx->strong;
    *n_dofs = P ? P->n : 0;
    *nnz = P ? P->nnz : 0;
    *n_classes = P ? P->n_classes : 0;
}

void strong_directions(const bt_ctx* ctx, int32_t* dir) {
    for (int d = 0; d < 3; ++d) dir[d] = ctx->strong ? ctx->strong->dir[d] : 0;
}

void free_strong(bt_ctx* ctx) {
    delete ctx->strong;
    ctx->strong = nullptr;
}

}  // namespace bt
