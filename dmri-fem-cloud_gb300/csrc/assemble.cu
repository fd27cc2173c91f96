// Coloured, atomic-free assembly of the P1 Bloch-Torrey matrices.
//
// Replaces FFC's tabulate_tensor kernels + PETSc insertion behind DOLFIN's
// assemble() of the theta-method forms (DmriFemLib.py:41-50, 58-145, 240-254).
// All integrands are polynomials of degree <= 3 per cell, so the closed forms
// below are the exact integrals FFC's degree-5 quadrature evaluates:
//   M_ij  = V/20 (1 + d_ij)                           mass
//   K_ij  = V g_i^T D g_j                             stiffness, D per cell
//   T_ij  = (1/T2) M_ij                               T2 decay
//   Jk_ij = V/60 (2 x_i + S) (i=j), V/120 (x_i + x_j + S) (i!=j),  S = sum x
//   R     = kappa int_F [u][v] on interface facets: +B on (a,a),(b,b), -B on
//           (a,b),(b,a), B_ij = kappa A/12 (1 + d_ij)   (icondition_wBC)
//           With a Crouzeix-Raviart kappa (the per-interface permeability of
//           MultilayeredDiskVariablePermeability.ipynb:480-502: the CR dof of a
//           facet is the region pair's value where the regions differ, else 0),
//           kappa is linear on each side of the facet, with vertex values
//           sum_g kappa_g - 3 kappa_opposite(v) (the P1 function whose face
//           centroids carry the four dofs), and avg() takes the mean of the two
//           sides: B_ij = A sum_l c_ijl kappa_l with c = 1/10 (i = j = l),
//           1/30 (two equal), 1/60 (all distinct), the exact cubic integral.
// Cells of one colour share no vertex, so one thread per cell adds its 4x4
// blocks straight into the CSR values without atomics; colours run in a fixed
// order, so every sum is formed in the same order on every run.  An interface
// facet is added by the lower-index cell of its pair, in that cell's colour
// pass: its rows belong to the owner cell's vertices, which no other cell of
// the colour touches.
#include "bt_common.cuh"

namespace bt {

namespace {

struct AsmArgs {
    const double* xyz;
    const int32_t* tets;
    const int32_t* region;
    const int32_t* comp;
    const int32_t* nbr;
    const int32_t* dof_of;
    const int32_t* row_ptr;
    const int32_t* col;
    const int32_t* cells;  // cells of this colour
    int32_t n_cells;
    int32_t nc;
    int32_t n_regions;
    const double* D_region;
    const double* D_cell;  // nullable, 6 per cell
    const double* invT2_region;
    const double* invT2_cell;  // nullable, 1 per cell (overrides invT2_region)
    const double* kappa_pair;
    int32_t kappa_cr;      // 1: Crouzeix-Raviart kappa (linear on each side of a facet)
    double *M, *K, *T, *R, *Jx, *Jy, *Jz, *w, *vw;
    int* status;
};

__device__ __forceinline__ int32_t find_pos(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                            int32_t row, int32_t c) {
    int32_t lo = row_ptr[row], hi = row_ptr[row + 1];
    while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        int32_t v = col[mid];
        if (v == c) return mid;
        if (v < c) lo = mid + 1; else hi = mid;
    }
    return -1;  // unreachable for a consistent graph
}

// CR dof of face k of cell c: the region pair's permeability when the cell
// across the face lies in another region, else 0 (boundary faces too).
__device__ __forceinline__ double cr_face_kappa(const AsmArgs& a, int32_t c, int k) {
    const int32_t n = a.nbr[(int64_t)c * 4 + k];
    if (n < 0) return 0.0;
    const int rc = a.region[c], rn = a.region[n];
    return (rc == rn) ? 0.0 : a.kappa_pair[rc * a.n_regions + rn];
}

__global__ void k_assemble_colour(AsmArgs a) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_cells) return;
    const int32_t t = a.cells[i];
    const int4 q = reinterpret_cast<const int4*>(a.tets)[t];
    const int32_t v[4] = {q.x, q.y, q.z, q.w};
    double X[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) X[k][c] = a.xyz[(int64_t)v[k] * 3 + c];
    double E[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) E[r][c] = X[r + 1][c] - X[0][c];
    // inverse of E via cofactors: Einv = adj(E)/det
    const double c00 = E[1][1] * E[2][2] - E[1][2] * E[2][1];
    const double c01 = E[1][2] * E[2][0] - E[1][0] * E[2][2];
    const double c02 = E[1][0] * E[2][1] - E[1][1] * E[2][0];
    const double det = E[0][0] * c00 + E[0][1] * c01 + E[0][2] * c02;
    const double id = 1.0 / det;
    double Ei[3][3];
    Ei[0][0] = c00 * id;
    Ei[1][0] = c01 * id;
    Ei[2][0] = c02 * id;
    Ei[0][1] = (E[0][2] * E[2][1] - E[0][1] * E[2][2]) * id;
    Ei[1][1] = (E[0][0] * E[2][2] - E[0][2] * E[2][0]) * id;
    Ei[2][1] = (E[0][1] * E[2][0] - E[0][0] * E[2][1]) * id;
    Ei[0][2] = (E[0][1] * E[1][2] - E[0][2] * E[1][1]) * id;
    Ei[1][2] = (E[0][2] * E[1][0] - E[0][0] * E[1][2]) * id;
    Ei[2][2] = (E[0][0] * E[1][1] - E[0][1] * E[1][0]) * id;
    // grad l_{k+1} = column k of Einv; grad l_0 = -(sum)
    double G[4][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        G[1][c] = Ei[c][0];
        G[2][c] = Ei[c][1];
        G[3][c] = Ei[c][2];
        G[0][c] = -(G[1][c] + G[2][c] + G[3][c]);
    }
    const double vol = fabs(det) / 6.0;
    const int reg = a.region[t];
    const int f = a.comp[t];
    double D[3][3];
    if (a.D_cell) {
        const double* d = a.D_cell + (int64_t)t * 6;
        D[0][0] = d[0]; D[1][1] = d[1]; D[2][2] = d[2];
        D[0][1] = D[1][0] = d[3];
        D[0][2] = D[2][0] = d[4];
        D[1][2] = D[2][1] = d[5];
    } else {
        const double s = a.D_region[reg];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) D[r][c] = (r == c) ? s : 0.0;
    }
    const double iT2 = a.invT2_cell ? a.invT2_cell[t] : a.invT2_region[reg];
    double DG[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int r = 0; r < 3; ++r) DG[k][r] = D[r][0] * G[k][0] + D[r][1] * G[k][1] + D[r][2] * G[k][2];
    double Sx[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) Sx[c] = X[0][c] + X[1][c] + X[2][c] + X[3][c];
    int32_t d[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) d[k] = a.dof_of[(int64_t)v[k] * a.nc + f];
    const double v20 = vol / 20.0, v60 = vol / 60.0, v120 = vol / 120.0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        a.w[d[r]] += 0.25 * vol;
        a.vw[v[r]] += 0.25 * vol;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int32_t p = find_pos(a.row_ptr, a.col, d[r], d[c]);
            if (p < 0) {  // inconsistent graph: record, never write out of bounds
                atomicCAS(a.status, DEV_OK, DEV_BAD_MESH);
                continue;
            }
            const double m = (r == c) ? 2.0 * v20 : v20;
            a.M[p] += m;
            a.K[p] += vol * (G[r][0] * DG[c][0] + G[r][1] * DG[c][1] + G[r][2] * DG[c][2]);
            a.T[p] += iT2 * m;
            if (r == c) {
                a.Jx[p] += v60 * (2.0 * X[r][0] + Sx[0]);
                a.Jy[p] += v60 * (2.0 * X[r][1] + Sx[1]);
                a.Jz[p] += v60 * (2.0 * X[r][2] + Sx[2]);
            } else {
                a.Jx[p] += v120 * (X[r][0] + X[c][0] + Sx[0]);
                a.Jy[p] += v120 * (X[r][1] + X[c][1] + Sx[1]);
                a.Jz[p] += v120 * (X[r][2] + X[c][2] + Sx[2]);
            }
        }
    }
    // interface facets owned by this cell
#pragma unroll
    for (int fa = 0; fa < 4; ++fa) {
        const int32_t nb = a.nbr[(int64_t)t * 4 + fa];
        if (nb <= t) continue;  // boundary (-1) or owned by the other cell
        const int g = a.comp[nb];
        if (g == f) continue;
        const double kap = a.kappa_pair[reg * a.n_regions + a.region[nb]];
        int fv[3], m = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k != fa) fv[m++] = k;
        double e1[3], e2[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            e1[c] = X[fv[1]][c] - X[fv[0]][c];
            e2[c] = X[fv[2]][c] - X[fv[0]][c];
        }
        const double cx = e1[1] * e2[2] - e1[2] * e2[1];
        const double cy = e1[2] * e2[0] - e1[0] * e2[2];
        const double cz = e1[0] * e2[1] - e1[1] * e2[0];
        const double area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
        const double b = kap * area / 12.0;
        // Crouzeix-Raviart kappa: the mean of both sides' vertex values on the facet
        double kv[3] = {0.0, 0.0, 0.0};
        if (a.kappa_cr) {
            double kt[4], kn[4], st = 0.0, sn = 0.0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                kt[k] = cr_face_kappa(a, t, k);
                kn[k] = cr_face_kappa(a, nb, k);
                st += kt[k];
                sn += kn[k];
            }
            const int4 qn = reinterpret_cast<const int4*>(a.tets)[nb];
            const int32_t vn[4] = {qn.x, qn.y, qn.z, qn.w};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double kb = 0.0;
#pragma unroll
                for (int l = 0; l < 4; ++l)
                    if (vn[l] == v[fv[k]]) kb = sn - 3.0 * kn[l];
                kv[k] = 0.5 * ((st - 3.0 * kt[fv[k]]) + kb);
            }
        }
        int32_t df[3], dg[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            df[k] = d[fv[k]];
            dg[k] = a.dof_of[(int64_t)v[fv[k]] * a.nc + g];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                double bb = (r == c) ? 2.0 * b : b;
                if (a.kappa_cr) {
                    bb = 0.0;
#pragma unroll
                    for (int l = 0; l < 3; ++l) {
                        const int ndist = (r == c) ? ((l == r) ? 1 : 2) : ((l == r || l == c) ? 2 : 3);
                        bb += area * (ndist == 1 ? 1.0 / 10.0 : (ndist == 2 ? 1.0 / 30.0 : 1.0 / 60.0)) * kv[l];
                    }
                }
                const int32_t p0 = find_pos(a.row_ptr, a.col, df[r], df[c]);
                const int32_t p1 = find_pos(a.row_ptr, a.col, dg[r], dg[c]);
                const int32_t p2 = find_pos(a.row_ptr, a.col, df[r], dg[c]);
                const int32_t p3 = find_pos(a.row_ptr, a.col, dg[r], df[c]);
                if ((p0 | p1 | p2 | p3) < 0) {
                    atomicCAS(a.status, DEV_OK, DEV_BAD_MESH);
                    continue;
                }
                a.R[p0] += bb;
                a.R[p1] += bb;
                a.R[p2] -= bb;
                a.R[p3] -= bb;
            }
    }
}

__global__ void k_partial_sum(const double* __restrict__ x, int64_t n, double* __restrict__ out, int nblocks) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)nblocks * blockDim.x)
        acc[0] += x[i];
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) out[blockIdx.x] = acc[0];
}

__global__ void k_partial_dot(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                              double* __restrict__ out, int nblocks) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)nblocks * blockDim.x)
        acc[0] += x[i] * y[i];
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) out[blockIdx.x] = acc[0];
}

}  // namespace

// Deterministic device sums (fixed grid, fixed order; final add on the host).
double device_sum(const double* d, int64_t n, cudaStream_t s) {
    const int nb = 256;
    DevBuf<double> part;
    part.alloc(nb);
    k_partial_sum<<<nb, 256, 0, s>>>(d, n, part, nb);
    BT_CUDA(cudaGetLastError());
    std::vector<double> h(nb);
    part.download(h.data(), nb, s);
    BT_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for (double v : h) t += v;
    return t;
}

double device_dot(const double* a, const double* b, int64_t n, cudaStream_t s) {
    const int nb = 256;
    DevBuf<double> part;
    part.alloc(nb);
    k_partial_dot<<<nb, 256, 0, s>>>(a, b, n, part, nb);
    BT_CUDA(cudaGetLastError());
    std::vector<double> h(nb);
    part.download(h.data(), nb, s);
    BT_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for (double v : h) t += v;
    return t;
}

void assemble_all(bt_ctx* ctx) {
    Mesh& m = ctx->mesh;
    Coeffs& cf = ctx->coeffs;
    Assembled& A = ctx->mat;
    cudaStream_t s = ctx->stream;
    BT_REQUIRE(m.built, BT_ERR_STATE, "bt_assemble: no mesh uploaded");
    BT_REQUIRE(cf.set, BT_ERR_STATE, "bt_assemble: coefficients not set");
    A.done = false;
    DevBuf<double>* mats[] = {&A.M, &A.K, &A.T, &A.R, &A.Jx, &A.Jy, &A.Jz};
    for (auto* b : mats) {
        b->alloc(m.nnz);
        b->zero(s);
    }
    A.w.alloc(m.n_dofs);
    A.w.zero(s);
    A.vw.alloc(m.n_v);
    A.vw.zero(s);
    AsmArgs a;
    a.xyz = m.xyz;
    a.tets = m.tets;
    a.region = m.region;
    a.comp = m.comp;
    a.nbr = m.nbr;
    a.dof_of = m.dof_of;
    a.row_ptr = m.row_ptr;
    a.col = m.col;
    a.nc = m.n_comp;
    a.n_regions = m.n_regions;
    a.D_region = cf.D_region;
    a.D_cell = cf.has_cell_D ? cf.D_cell.p : nullptr;
    a.invT2_region = cf.invT2_region;
    a.invT2_cell = cf.has_cell_T2 ? cf.invT2_cell.p : nullptr;
    a.kappa_pair = cf.kappa_pair;
    a.kappa_cr = cf.kappa_cr ? 1 : 0;
    a.M = A.M; a.K = A.K; a.T = A.T; a.R = A.R;
    a.Jx = A.Jx; a.Jy = A.Jy; a.Jz = A.Jz;
    a.w = A.w;
    a.vw = A.vw;
    DevBuf<int> status;
    status.alloc(1);
    status.zero(s);
    a.status = status;
    for (int c = 0; c < m.n_colours; ++c) {
        const int32_t b = m.colour_ptr[c], e = m.colour_ptr[c + 1];
        if (e <= b) continue;
        a.cells = m.colour_cells.p + b;
        a.n_cells = e - b;
        k_assemble_colour<<<(unsigned)((a.n_cells + 127) / 128), 128, 0, s>>>(a);
        BT_CUDA(cudaGetLastError());
    }
    int st = 0;
    BT_CUDA(cudaMemcpyAsync(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    BT_CUDA(cudaStreamSynchronize(s));
    BT_REQUIRE(st == DEV_OK, BT_ERR_INVALID, "bt_assemble: a cell coupling is missing from the graph");
    m.volume = device_sum(A.vw, m.n_v, s);
    A.done = true;
    ++A.version;
}

}  // namespace bt
