// Weak pseudo-periodic boundary conditions: the host-side set-up.
//
// Reference: the weak ("penalty") form of DmriFemLib.py, used when
// mydomain.PeriodicDir != [0,0,0] and IsDomainPeriodic is False:
//   * ThetaMethodF_wBC1c/2c (DmriFemLib.py:79-93, 125-145) add to the implicit
//     form  theta kappa_e (ur vr + ui vi) ds  (2c: weighted by the cell's phase);
//   * ThetaMethodL_wBC1c/2c (DmriFemLib.py:58-77, 96-122) add to the explicit
//     form  (1-theta) kappa_e (ubc_r vr + ubc_i vi) ds, with ubc the
//     WeakPseudoPeriodic_1c/2c expression (DmriFemLib.py:256-323, 386-451):
//     at a point x on a periodic face it is u_n at the mirror point on the
//     opposite face, rotated by exp(i q F(tp) g.ln) with ln the shift to the
//     mirror point; elsewhere 0;
//   * kappa_e = (3e-3 / hmin) * [x within 1e-2 hmin of a periodic face]
//     (WeakPseudoPeridicMarker, DmriFemLib.py:598-610; hmin = the smallest cell
//     diameter, DmriFemLib.py:587-589).
// Both kappa_e and ubc are degree-1 expressions, i.e. P1 interpolants on each
// cell, so the facet integrals are exact cubic integrals on triangles:
//     int_F l_a l_b l_c = |F|/10 (a=b=c), |F|/30 (two equal), |F|/60 (distinct).
// The mirror point of a vertex follows the reference's eval order: directions
// x, y, z; in each the min face, then the max face (tolerance 1e-7); a later
// match replaces an earlier one.  Its value is the P1 interpolant on the
// boundary triangle of the opposite face that contains it (the closest one when
// none does, as DOLFIN's allow_extrapolation evaluation), taken from the dofs
// of the boundary vertex's own compartment (a vertex of that triangle with no
// dof in the compartment contributes zero).
#include "bt_common.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

namespace bt {

namespace {

struct Mirror {
    bool on = false;
    double shift[3] = {0.0, 0.0, 0.0};
    int32_t w[3] = {-1, -1, -1};   // vertices of the mirror triangle
    double lam[3] = {0.0, 0.0, 0.0};
};

inline double tri3(int a, int b, int c) {
    if (a == b && b == c) return 1.0 / 10.0;
    if (a == b || b == c || a == c) return 1.0 / 30.0;
    return 1.0 / 60.0;
}

// Boundary triangles of one plane, bucketed on a uniform 2D grid (axes u, v).
struct PlaneIndex {
    int au = 0, av = 0;
    double u0 = 0, v0 = 0, hu = 1, hv = 1;
    int nu = 1, nv = 1;
    std::vector<std::array<int32_t, 3>> tri;
    std::vector<int32_t> cell_ptr, cell_tri;

    void build(const std::vector<double>& xyz, int d) {
        au = (d + 1) % 3;
        av = (d + 2) % 3;
        if (tri.empty()) return;
        double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300};
        for (auto& t : tri)
            for (int k = 0; k < 3; ++k) {
                const double p[2] = {xyz[3 * (size_t)t[k] + au], xyz[3 * (size_t)t[k] + av]};
                for (int c = 0; c < 2; ++c) {
                    lo[c] = std::min(lo[c], p[c]);
                    hi[c] = std::max(hi[c], p[c]);
                }
            }
        const int side = std::max(1, (int)std::sqrt((double)tri.size() / 2.0));
        nu = nv = side;
        u0 = lo[0];
        v0 = lo[1];
        hu = std::max((hi[0] - lo[0]) / nu, 1e-300);
        hv = std::max((hi[1] - lo[1]) / nv, 1e-300);
        std::vector<int32_t> cnt((size_t)nu * nv + 1, 0);
        auto cells_of = [&](const std::array<int32_t, 3>& t, int& i0, int& i1, int& j0, int& j1) {
            double a0 = 1e300, a1 = -1e300, b0 = 1e300, b1 = -1e300;
            for (int k = 0; k < 3; ++k) {
                a0 = std::min(a0, xyz[3 * (size_t)t[k] + au]);
                a1 = std::max(a1, xyz[3 * (size_t)t[k] + au]);
                b0 = std::min(b0, xyz[3 * (size_t)t[k] + av]);
                b1 = std::max(b1, xyz[3 * (size_t)t[k] + av]);
            }
            i0 = clampi((int)std::floor((a0 - u0) / hu), nu);
            i1 = clampi((int)std::floor((a1 - u0) / hu), nu);
            j0 = clampi((int)std::floor((b0 - v0) / hv), nv);
            j1 = clampi((int)std::floor((b1 - v0) / hv), nv);
        };
        for (auto& t : tri) {
            int i0, i1, j0, j1;
            cells_of(t, i0, i1, j0, j1);
            for (int i = i0; i <= i1; ++i)
                for (int j = j0; j <= j1; ++j) ++cnt[(size_t)i * nv + j + 1];
        }
        for (size_t c = 1; c < cnt.size(); ++c) cnt[c] += cnt[c - 1];
        cell_ptr = cnt;
        cell_tri.assign(cnt.back(), 0);
        std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
        for (int32_t f = 0; f < (int32_t)tri.size(); ++f) {
            int i0, i1, j0, j1;
            cells_of(tri[f], i0, i1, j0, j1);
            for (int i = i0; i <= i1; ++i)
                for (int j = j0; j <= j1; ++j) cell_tri[fill[(size_t)i * nv + j]++] = f;
        }
    }
    static int clampi(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

    // barycentric coordinates of p (2D) in triangle f; returns min coordinate
    double bary(const std::vector<double>& xyz, int32_t f, const double p[2], double lam[3]) const {
        const auto& t = tri[f];
        const double ax = xyz[3 * (size_t)t[0] + au], ay = xyz[3 * (size_t)t[0] + av];
        const double bx = xyz[3 * (size_t)t[1] + au], by = xyz[3 * (size_t)t[1] + av];
        const double cx = xyz[3 * (size_t)t[2] + au], cy = xyz[3 * (size_t)t[2] + av];
        const double det = (bx - ax) * (cy - ay) - (cx - ax) * (by - ay);
        if (std::fabs(det) < 1e-300) {
            lam[0] = lam[1] = lam[2] = 0.0;
            return -1e300;
        }
        lam[1] = ((p[0] - ax) * (cy - ay) - (cx - ax) * (p[1] - ay)) / det;
        lam[2] = ((bx - ax) * (p[1] - ay) - (p[0] - ax) * (by - ay)) / det;
        lam[0] = 1.0 - lam[1] - lam[2];
        return std::min(lam[0], std::min(lam[1], lam[2]));
    }

    // the triangle containing p (largest smallest coordinate); all triangles
    // are searched when the grid cell has no containing one
    bool locate(const std::vector<double>& xyz, const double pt[3], int32_t w[3], double lam[3]) const {
        if (tri.empty()) return false;
        const double p[2] = {pt[au], pt[av]};
        double best = -1e300, bl[3] = {0, 0, 0};
        int32_t bf = -1;
        auto scan = [&](int32_t f) {
            double l[3];
            const double mn = bary(xyz, f, p, l);
            if (mn > best) {
                best = mn;
                bf = f;
                bl[0] = l[0]; bl[1] = l[1]; bl[2] = l[2];
            }
        };
        const int i = clampi((int)std::floor((p[0] - u0) / hu), nu), j = clampi((int)std::floor((p[1] - v0) / hv), nv);
        for (int32_t e = cell_ptr[(size_t)i * nv + j]; e < cell_ptr[(size_t)i * nv + j + 1]; ++e) scan(cell_tri[e]);
        if (best < -1e-9)
            for (int32_t f = 0; f < (int32_t)tri.size(); ++f) scan(f);
        if (bf < 0) return false;
        for (int k = 0; k < 3; ++k) {
            w[k] = tri[bf][k];
            lam[k] = bl[k];
        }
        return best >= -1e-6;
    }
};

}  // namespace

void set_periodic(bt_ctx* ctx, const int32_t* dir) {
    Mesh& m = ctx->mesh;
    Periodic& P = ctx->per;
    cudaStream_t s = ctx->stream;
    P.on = false;
    P.PB.release();
    P.ptr.release();
    P.col.release();
    P.val.release();
    P.n_facets = P.n_rows = P.n_entries = P.n_unmatched = 0;
    for (int d = 0; d < 3; ++d) {
        BT_REQUIRE(dir[d] == 0 || dir[d] == 1, BT_ERR_INVALID, "periodic directions must be 0 or 1");
        P.dir[d] = dir[d];
    }
    if (!dir[0] && !dir[1] && !dir[2]) return;
    const int64_t n_v = m.n_v, n_t = m.n_t, nc = m.n_comp, n = m.n_dofs;
    std::vector<double> xyz((size_t)n_v * 3);
    std::vector<int32_t> tets((size_t)n_t * 4), comp((size_t)n_t), nbr((size_t)n_t * 4), dof_of((size_t)n_v * nc),
        rp((size_t)n + 1), col((size_t)m.nnz), dvert((size_t)n), dcomp((size_t)n);
    m.xyz.download(xyz.data(), xyz.size(), s);
    m.tets.download(tets.data(), tets.size(), s);
    m.comp.download(comp.data(), comp.size(), s);
    m.nbr.download(nbr.data(), nbr.size(), s);
    m.dof_of.download(dof_of.data(), dof_of.size(), s);
    m.row_ptr.download(rp.data(), rp.size(), s);
    m.col.download(col.data(), col.size(), s);
    m.dof_vertex.download(dvert.data(), dvert.size(), s);
    m.dof_comp.download(dcomp.data(), dcomp.size(), s);
    BT_CUDA(cudaStreamSynchronize(s));

    // bounding box; hmin = smallest cell diameter (largest vertex distance of a cell)
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
    BT_REQUIRE(hmin > 0.0 && std::isfinite(hmin), BT_ERR_INVALID, "periodic set-up: degenerate mesh");
    const double eps = 1e-2 * hmin, ks = 3e-3 / hmin, tol = 1e-7;
    P.hmin = hmin;
    P.kappa_e = ks;

    // kappa_e at the vertices
    std::vector<double> kap((size_t)n_v, 0.0);
    for (int64_t v = 0; v < n_v; ++v) {
        bool on = false;
        for (int d = 0; d < 3; ++d)
            on = on || (dir[d] && (xyz[3 * v + d] < lo[d] + eps || xyz[3 * v + d] > hi[d] - eps));
        kap[v] = on ? ks : 0.0;
    }

    // exterior facets (local vertex a opposite the facet), and the triangles
    // lying on each face of the box
    std::vector<std::array<int32_t, 4>> facets;   // cell, three vertices
    PlaneIndex plane[3][2];
    for (int64_t t = 0; t < n_t; ++t)
        for (int a = 0; a < 4; ++a) {
            if (nbr[4 * t + a] >= 0) continue;
            std::array<int32_t, 3> f;
            int k = 0;
            for (int b = 0; b < 4; ++b)
                if (b != a) f[k++] = tets[4 * t + b];
            facets.push_back({(int32_t)t, f[0], f[1], f[2]});
            for (int d = 0; d < 3; ++d)
                for (int sd = 0; sd < 2; ++sd) {
                    const double pl = sd ? hi[d] : lo[d];
                    bool on = true;
                    for (int q = 0; q < 3; ++q) on = on && std::fabs(xyz[3 * (size_t)f[q] + d] - pl) <= eps;
                    if (on && dir[d]) plane[d][sd].tri.push_back(f);
                }
        }
    for (int d = 0; d < 3; ++d)
        for (int sd = 0; sd < 2; ++sd) plane[d][sd].build(xyz, d);

    // mirror points (reference eval order; a later match replaces an earlier one)
    std::vector<Mirror> mir((size_t)n_v);
    for (int64_t v = 0; v < n_v; ++v) {
        int md = -1, ms = 0;
        for (int d = 0; d < 3; ++d) {
            if (!dir[d]) continue;
            if (std::fabs(xyz[3 * v + d] - lo[d]) <= tol) { md = d; ms = 1; }
            if (std::fabs(xyz[3 * v + d] - hi[d]) <= tol) { md = d; ms = 0; }
        }
        if (md < 0) continue;
        Mirror& M = mir[v];
        double pt[3] = {xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]};
        pt[md] = ms ? hi[md] : lo[md];
        M.shift[md] = pt[md] - xyz[3 * v + md];
        M.on = true;
        if (!plane[md][ms].locate(xyz, pt, M.w, M.lam)) ++P.n_unmatched;
        if (M.w[0] < 0) M.on = false;
        for (int k = 0; k < 3; ++k)
            if (std::fabs(M.lam[k]) <= 1e-13) M.lam[k] = 0.0;
    }

    // PB: kappa_e-weighted facet mass of the facet's compartment dofs (CSR order)
    auto csr_pos = [&](int32_t i, int32_t j) -> int64_t {
        const int32_t* b = col.data() + rp[i];
        const int32_t* e = col.data() + rp[i + 1];
        const int32_t* it = std::lower_bound(b, e, j);
        BT_REQUIRE(it != e && *it == j, BT_ERR_INVALID, "periodic set-up: facet pair outside the sparsity");
        return (int64_t)(it - col.data());
    };
    std::vector<double> pb((size_t)m.nnz, 0.0);
    for (const auto& f : facets) {
        const int32_t c = comp[f[0]];
        const double ka[3] = {kap[f[1]], kap[f[2]], kap[f[3]]};
        if (ka[0] == 0.0 && ka[1] == 0.0 && ka[2] == 0.0) continue;
        double e1[3], e2[3];
        for (int d = 0; d < 3; ++d) {
            e1[d] = xyz[3 * (size_t)f[2] + d] - xyz[3 * (size_t)f[1] + d];
            e2[d] = xyz[3 * (size_t)f[3] + d] - xyz[3 * (size_t)f[1] + d];
        }
        const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                     cz = e1[0] * e2[1] - e1[1] * e2[0];
        const double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
        int32_t dd[3];
        for (int k = 0; k < 3; ++k) {
            dd[k] = dof_of[(size_t)f[1 + k] * nc + c];
            BT_REQUIRE(dd[k] >= 0, BT_ERR_INVALID, "periodic set-up: facet vertex without a dof");
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double v = 0.0;
                for (int a = 0; a < 3; ++a) v += ka[a] * tri3(a, i, j);
                pb[csr_pos(dd[i], dd[j])] += area * v;
            }
        ++P.n_facets;
    }

    // explicit entries: row i, over its PB columns j with a mirror, over the
    // mirror triangle's dofs k of j's compartment
    std::vector<int32_t> hptr((size_t)n + 1, 0), hcol;
    std::vector<PerVal> hval;
    for (int64_t i = 0; i < n; ++i) {
        for (int32_t e = rp[i]; e < rp[i + 1]; ++e) {
            if (pb[e] == 0.0) continue;
            const int32_t j = col[e];
            const Mirror& M = mir[dvert[j]];
            if (!M.on) continue;
            for (int k = 0; k < 3; ++k) {
                if (M.lam[k] == 0.0) continue;
                const int32_t dk = dof_of[(size_t)M.w[k] * nc + dcomp[j]];
                if (dk < 0) continue;
                hcol.push_back(dk);
                hval.push_back(PerVal{pb[e] * M.lam[k], M.shift[0], M.shift[1], M.shift[2]});
            }
        }
        hptr[i + 1] = (int32_t)hcol.size();
        if (hptr[i + 1] > hptr[i]) ++P.n_rows;
    }
    BT_REQUIRE(hcol.size() < (size_t)INT32_MAX, BT_ERR_INVALID, "periodic set-up: too many boundary entries");
    P.n_entries = (int64_t)hcol.size();
    P.PB.upload(pb.data(), pb.size(), s);
    P.ptr.upload(hptr.data(), hptr.size(), s);
    if (!hcol.empty()) {
        P.col.upload(hcol.data(), hcol.size(), s);
        P.val.upload(hval.data(), hval.size(), s);
    }
    BT_CUDA(cudaStreamSynchronize(s));
    P.on = true;
}

}  // namespace bt
