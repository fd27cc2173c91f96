// Device builder of the duplicated-interface-node graph of a P1 tetrahedral mesh.
//
// The reference carries two fields on the whole mesh and lets `ident_zeros`
// pin the rows of vertices that touch no cell of a field
// (DmriFemLib.py:240-254, 459-463).  Here every live (vertex, compartment) pair
// is one complex dof, numbered vertex-major, so interface vertices appear once
// per side; the coupling of the two sides across interface facets
// (icondition_wBC, DmriFemLib.py:47-50) adds the cross-compartment entries.
//
// Steps (all on the device, deterministic):
//   1. live flags and dof numbering (exclusive scan);
//   2. vertex -> cell incidence lists, sorted;
//   3. face neighbours (cell across each face) from the incidence lists;
//   4. CSR rows: sorted unique columns per dof (count pass + fill pass);
//   5. Jones-Plassmann cell colouring (no two cells of a colour share a vertex),
//      used by the atomic-free assembly kernel;
//   6. sliced ELL (C = 32 rows per slice, column-major inside a slice) for the
//      coalesced single-RHS SpMV of the stepper.
#include "bt_common.cuh"

#include <algorithm>

namespace bt {

namespace {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;
constexpr int kMaxRow = 160;  // unique columns per dof row

__global__ void k_scan_tiles(const int32_t* __restrict__ in, int32_t* __restrict__ out,
                             int32_t* __restrict__ tile_sums, int64_t n) {
    __shared__ int32_t sh[kScanBlock];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int32_t run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        int32_t x = (i < n) ? in[i] : 0;
        v[k] = run;
        run += x;
    }
    sh[threadIdx.x] = run;
    __syncthreads();
    // Hillis-Steele over the 256 thread totals
    for (int o = 1; o < kScanBlock; o <<= 1) {
        int32_t t = (threadIdx.x >= (unsigned)o) ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    int32_t excl = sh[threadIdx.x] - run;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = v[k] + excl;
    }
    if (threadIdx.x == kScanBlock - 1) tile_sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void k_scan_add(int32_t* __restrict__ out, const int32_t* __restrict__ tile_off, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_off[i / kScanTile];
}

}  // namespace

// Exclusive prefix sum of int32 (n >= 1); *total_out (host) receives the sum.
void exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int32_t* total_out,
                        cudaStream_t s) {
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    DevBuf<int32_t> sums, offs;
    sums.alloc(tiles);
    offs.alloc(tiles);
    k_scan_tiles<<<(unsigned)tiles, kScanBlock, 0, s>>>(in, out, sums, n);
    BT_CUDA(cudaGetLastError());
    if (tiles > 1) {
        int32_t t2 = 0;
        exclusive_scan_i32(sums, offs, tiles, &t2, s);
        k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, offs, n);
        BT_CUDA(cudaGetLastError());
    }
    if (total_out) {
        int32_t last_in = 0, last_out = 0;
        BT_CUDA(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        BT_CUDA(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        BT_CUDA(cudaStreamSynchronize(s));
        int64_t tot = (int64_t)last_in + (int64_t)last_out;
        BT_REQUIRE(tot <= INT32_MAX, BT_ERR_INVALID, "prefix sum overflows int32");
        *total_out = (int32_t)tot;
    }
}

namespace {

__global__ void k_mark_live(const int32_t* __restrict__ tets, const int32_t* __restrict__ comp,
                            int64_t n_t, int nc, int32_t* __restrict__ live) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_t) return;
    const int f = comp[t];
#pragma unroll
    for (int a = 0; a < 4; ++a) live[(int64_t)tets[t * 4 + a] * nc + f] = 1;
}

__global__ void k_number_dofs(const int32_t* __restrict__ live, const int32_t* __restrict__ scan,
                              int64_t n, int nc, int32_t* __restrict__ dof_of,
                              int32_t* __restrict__ dof_vertex, int32_t* __restrict__ dof_comp) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (live[i]) {
        const int32_t d = scan[i];
        dof_of[i] = d;
        dof_vertex[d] = (int32_t)(i / nc);
        dof_comp[d] = (int32_t)(i % nc);
    } else {
        dof_of[i] = -1;
    }
}

__global__ void k_count_vt(const int32_t* __restrict__ tets, int64_t n_t, int32_t* __restrict__ cnt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_t * 4) return;
    atomicAdd(&cnt[tets[i]], 1);
}

__global__ void k_fill_vt(const int32_t* __restrict__ tets, int64_t n_t, const int32_t* __restrict__ ptr,
                          int32_t* __restrict__ cursor, int32_t* __restrict__ list) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_t * 4) return;
    const int32_t v = tets[i];
    const int32_t k = atomicAdd(&cursor[v], 1);
    list[ptr[v] + k] = (int32_t)(i >> 2);
}

__global__ void k_sort_vt(const int32_t* __restrict__ ptr, int64_t n_v, int32_t* __restrict__ list) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_v) return;
    const int32_t b = ptr[v], e = ptr[v + 1];
    for (int32_t i = b + 1; i < e; ++i) {
        int32_t x = list[i];
        int32_t j = i - 1;
        while (j >= b && list[j] > x) {
            list[j + 1] = list[j];
            --j;
        }
        list[j + 1] = x;
    }
}

__device__ __forceinline__ bool cell_has(const int32_t* __restrict__ tets, int32_t c, int32_t v) {
    const int4 q = reinterpret_cast<const int4*>(tets)[c];
    return q.x == v || q.y == v || q.z == v || q.w == v;
}

// nbr[t*4+a] = cell sharing the face of t opposite its local vertex a, or -1.
__global__ void k_face_nbr(const int32_t* __restrict__ tets, int64_t n_t, const int32_t* __restrict__ vt_ptr,
                           const int32_t* __restrict__ vt_list, int32_t* __restrict__ nbr,
                           int* __restrict__ status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_t * 4) return;
    const int32_t t = (int32_t)(i >> 2);
    const int a = (int)(i & 3);
    int32_t fv[3];
    int m = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k != a) fv[m++] = tets[(int64_t)t * 4 + k];
    int32_t found = -1;
    int nfound = 0;
    for (int32_t e = vt_ptr[fv[0]]; e < vt_ptr[fv[0] + 1]; ++e) {
        const int32_t c = vt_list[e];
        if (c == t) continue;
        if (cell_has(tets, c, fv[1]) && cell_has(tets, c, fv[2])) {
            found = c;
            ++nfound;
        }
    }
    if (nfound > 1) atomicCAS(status, DEV_OK, DEV_BAD_MESH);  // non-manifold face
    nbr[i] = found;
}

// Insert x into the sorted unique list u[0..n); returns the new length.
__device__ __forceinline__ int sorted_insert(int32_t* u, int n, int32_t x, int* overflow) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (u[mid] < x) lo = mid + 1; else hi = mid;
    }
    if (lo < n && u[lo] == x) return n;
    if (n >= kMaxRow) {
        *overflow = 1;
        return n;
    }
    for (int j = n; j > lo; --j) u[j] = u[j - 1];
    u[lo] = x;
    return n + 1;
}

// Columns of dof d = (v, f): dofs (w, f) of every cell of compartment f that
// contains v, and dofs (w, g) of every interface facet through v whose other
// side lies in compartment g.
template <bool kFill>
__global__ void k_rows(const int32_t* __restrict__ tets, const int32_t* __restrict__ comp,
                       const int32_t* __restrict__ nbr, const int32_t* __restrict__ vt_ptr,
                       const int32_t* __restrict__ vt_list, const int32_t* __restrict__ dof_of,
                       const int32_t* __restrict__ dof_vertex, const int32_t* __restrict__ dof_comp,
                       int64_t n_dofs, int nc, int32_t* __restrict__ row_len,
                       const int32_t* __restrict__ row_ptr, int32_t* __restrict__ col,
                       int* __restrict__ status) {
    const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n_dofs) return;
    const int32_t v = dof_vertex[d];
    const int f = dof_comp[d];
    int32_t u[kMaxRow];
    int n = 0, overflow = 0;
    for (int32_t e = vt_ptr[v]; e < vt_ptr[v + 1]; ++e) {
        const int32_t c = vt_list[e];
        if (comp[c] != f) continue;
        const int4 q = reinterpret_cast<const int4*>(tets)[c];
        const int32_t cv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) n = sorted_insert(u, n, dof_of[(int64_t)cv[k] * nc + f], &overflow);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (cv[a] == v) continue;  // face opposite a must contain v
            const int32_t nb = nbr[(int64_t)c * 4 + a];
            if (nb < 0) continue;
            const int g = comp[nb];
            if (g == f) continue;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k != a) n = sorted_insert(u, n, dof_of[(int64_t)cv[k] * nc + g], &overflow);
        }
    }
    if (overflow) atomicCAS(status, DEV_OK, DEV_OVERFLOW);
    if (!kFill) {
        row_len[d] = n;
    } else {
        const int32_t b = row_ptr[d];
        for (int k = 0; k < n; ++k) col[b + k] = u[k];
    }
}

__global__ void k_diag_pos(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                           int64_t n, int32_t* __restrict__ diag_pos, int* __restrict__ status) {
    const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    int32_t lo = row_ptr[d], hi = row_ptr[d + 1];
    int32_t p = -1;
    while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        int32_t c = col[mid];
        if (c == (int32_t)d) { p = mid; break; }
        if (c < (int32_t)d) lo = mid + 1; else hi = mid;
    }
    if (p < 0) atomicCAS(status, DEV_OK, DEV_BAD_MESH);
    diag_pos[d] = p;
}

__device__ __forceinline__ uint32_t cell_priority(uint32_t t) {
    // integer hash (Wang-style mix); ties broken by the cell index
    uint32_t x = t * 0x9E3779B1u + 0x7F4A7C15u;
    x ^= x >> 16;
    x *= 0x85EBCA6Bu;
    x ^= x >> 13;
    x *= 0xC2B2AE35u;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ bool prio_gt(uint32_t pa, int32_t a, uint32_t pb, int32_t b) {
    return pa > pb || (pa == pb && a > b);
}

// Jones-Plassmann round, phase 1: select uncoloured cells whose priority is the
// largest among their uncoloured vertex-neighbours.  Reads only colours of
// earlier rounds.
__global__ void k_jp_select(const int32_t* __restrict__ tets, int64_t n_t, const int32_t* __restrict__ vt_ptr,
                            const int32_t* __restrict__ vt_list, const int32_t* __restrict__ colour,
                            int32_t* __restrict__ selected) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_t) return;
    const int32_t t = (int32_t)i;
    if (colour[t] >= 0) {
        selected[t] = 0;
        return;
    }
    const uint32_t pt = cell_priority((uint32_t)t);
    const int4 q = reinterpret_cast<const int4*>(tets)[t];
    const int32_t cv[4] = {q.x, q.y, q.z, q.w};
    int sel = 1;
    for (int a = 0; a < 4 && sel; ++a) {
        for (int32_t e = vt_ptr[cv[a]]; e < vt_ptr[cv[a] + 1]; ++e) {
            const int32_t c = vt_list[e];
            if (c == t || colour[c] >= 0) continue;
            if (prio_gt(cell_priority((uint32_t)c), c, pt, t)) {
                sel = 0;
                break;
            }
        }
    }
    selected[t] = sel;
}

// Phase 2: every selected cell takes the smallest colour unused by its
// neighbours.  No two selected cells are neighbours, so the colours read are
// final.
__global__ void k_jp_colour(const int32_t* __restrict__ tets, int64_t n_t, const int32_t* __restrict__ vt_ptr,
                            const int32_t* __restrict__ vt_list, const int32_t* __restrict__ selected,
                            int32_t* __restrict__ colour, int32_t* __restrict__ remaining,
                            int* __restrict__ status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_t) return;
    const int32_t t = (int32_t)i;
    if (!selected[t]) {
        if (colour[t] < 0) atomicAdd(remaining, 1);
        return;
    }
    uint32_t used[kMaxColours / 32];
#pragma unroll
    for (int k = 0; k < kMaxColours / 32; ++k) used[k] = 0u;
    const int4 q = reinterpret_cast<const int4*>(tets)[t];
    const int32_t cv[4] = {q.x, q.y, q.z, q.w};
    for (int a = 0; a < 4; ++a) {
        for (int32_t e = vt_ptr[cv[a]]; e < vt_ptr[cv[a] + 1]; ++e) {
            const int32_t c = colour[vt_list[e]];
            if (c >= 0) used[c >> 5] |= 1u << (c & 31);
        }
    }
    int pick = -1;
    for (int k = 0; k < kMaxColours / 32 && pick < 0; ++k) {
        if (used[k] != 0xffffffffu) pick = k * 32 + __ffs(~used[k]) - 1;
    }
    if (pick < 0) {
        atomicCAS(status, DEV_OK, DEV_OVERFLOW);
        pick = kMaxColours - 1;
    }
    colour[t] = pick;
}

__global__ void k_slice_width(const int32_t* __restrict__ row_ptr, int64_t n, int32_t n_slices,
                              int32_t* __restrict__ width, int32_t* __restrict__ entries) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_slices) return;
    int32_t w = 0;
    for (int k = 0; k < 32; ++k) {
        int64_t r = s * 32 + k;
        if (r < n) w = max(w, row_ptr[r + 1] - row_ptr[r]);
    }
    width[s] = w;
    entries[s] = w * 32;
}

__global__ void k_slice_fill(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col, int64_t n,
                             int32_t n_slices, const int32_t* __restrict__ sl_ptr,
                             const int32_t* __restrict__ sl_w, int32_t* __restrict__ sl_col,
                             int32_t* __restrict__ sl_pos) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_slices * 32) return;
    const int32_t s = (int32_t)(i >> 5);
    const int lane = (int)(i & 31);
    const int64_t r = i;
    const int32_t w = sl_w[s];
    const int32_t base = sl_ptr[s];
    int32_t b = 0, len = 0;
    if (r < n) {
        b = row_ptr[r];
        len = row_ptr[r + 1] - b;
    }
    for (int k = 0; k < w; ++k) {
        const int32_t e = base + k * 32 + lane;
        if (k < len) {
            sl_col[e] = col[b + k];
            sl_pos[e] = b + k;
        } else {
            sl_col[e] = (int32_t)r;  // padding: own row, zero value
            sl_pos[e] = -1;
        }
    }
}

inline unsigned nblk(int64_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }

void check_status(const int* d_status, cudaStream_t s, const char* what) {
    int st = 0;
    BT_CUDA(cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    BT_CUDA(cudaStreamSynchronize(s));
    if (st == DEV_BAD_MESH)
        throw Error(BT_ERR_INVALID, std::string(what) + ": invalid mesh (non-manifold face or missing diagonal)");
    if (st == DEV_OVERFLOW)
        throw Error(BT_ERR_INVALID, std::string(what) + ": vertex degree above the builder's limit");
    if (st != DEV_OK) throw Error(BT_ERR_CUDA, std::string(what) + ": device status " + std::to_string(st));
}

}  // namespace

void build_graph(bt_ctx* ctx, const double* xyz, int64_t n_v, const int32_t* tets, int64_t n_t,
                 const int32_t* region, int32_t n_regions, const int32_t* region_comp) {
    cudaStream_t s = ctx->stream;
    Mesh& m = ctx->mesh;
    m.built = false;
    BT_REQUIRE(n_v >= 4 && n_t >= 1, BT_ERR_INVALID, "mesh needs at least one tetrahedron");
    BT_REQUIRE(n_v < INT32_MAX && n_t * 4 < INT32_MAX, BT_ERR_INVALID, "mesh too large for int32 indices");
    BT_REQUIRE(n_regions >= 1, BT_ERR_INVALID, "n_regions must be >= 1");
    // host-side validation of indices
    std::vector<int32_t> rc(n_regions);
    int32_t nc = 0;
    for (int32_t r = 0; r < n_regions; ++r) {
        rc[r] = region_comp ? region_comp[r] : (r % 2);
        BT_REQUIRE(rc[r] >= 0 && rc[r] < kMaxCompartments, BT_ERR_INVALID, "compartment id out of range [0,8)");
    }
    std::vector<int32_t> comp(n_t);
    std::vector<char> comp_used(kMaxCompartments, 0);
    for (int64_t t = 0; t < n_t; ++t) {
        for (int a = 0; a < 4; ++a) {
            int32_t v = tets[t * 4 + a];
            BT_REQUIRE(v >= 0 && v < n_v, BT_ERR_INVALID, "tet vertex index out of range");
        }
        const int32_t r = region[t];
        BT_REQUIRE(r >= 0 && r < n_regions, BT_ERR_INVALID, "cell region out of range");
        comp[t] = rc[r];
        comp_used[rc[r]] = 1;
    }
    for (int f = 0; f < kMaxCompartments; ++f)
        if (comp_used[f]) nc = f + 1;
    m.n_v = n_v;
    m.n_t = n_t;
    m.n_regions = n_regions;
    m.n_comp = nc;
    m.region_comp = rc;
    m.xyz.upload(xyz, n_v * 3, s);
    m.tets.upload(tets, n_t * 4, s);
    m.region.upload(region, n_t, s);
    m.comp.upload(comp.data(), n_t, s);

    DevBuf<int> status;
    status.alloc(1);
    status.zero(s);

    // 1. live flags and dof numbering
    const int64_t nvc = n_v * nc;
    DevBuf<int32_t> live, scan;
    live.alloc(nvc);
    live.zero(s);
    scan.alloc(nvc);
    k_mark_live<<<nblk(n_t), 256, 0, s>>>(m.tets, m.comp, n_t, nc, live);
    BT_CUDA(cudaGetLastError());
    int32_t n_dofs = 0;
    exclusive_scan_i32(live, scan, nvc, &n_dofs, s);
    m.n_dofs = n_dofs;
    m.dof_of.alloc(nvc);
    m.dof_vertex.alloc(n_dofs);
    m.dof_comp.alloc(n_dofs);
    k_number_dofs<<<nblk(nvc), 256, 0, s>>>(live, scan, nvc, nc, m.dof_of, m.dof_vertex, m.dof_comp);
    BT_CUDA(cudaGetLastError());

    // 2. vertex -> cell incidence
    DevBuf<int32_t> cnt, cursor;
    cnt.alloc(n_v + 1);
    cnt.zero(s);
    k_count_vt<<<nblk(n_t * 4), 256, 0, s>>>(m.tets, n_t, cnt);
    BT_CUDA(cudaGetLastError());
    m.vt_ptr.alloc(n_v + 1);
    int32_t tot = 0;
    exclusive_scan_i32(cnt, m.vt_ptr, n_v + 1, &tot, s);
    m.vt_list.alloc(n_t * 4);
    cursor.alloc(n_v);
    cursor.zero(s);
    k_fill_vt<<<nblk(n_t * 4), 256, 0, s>>>(m.tets, n_t, m.vt_ptr, cursor, m.vt_list);
    k_sort_vt<<<nblk(n_v), 256, 0, s>>>(m.vt_ptr, n_v, m.vt_list);
    BT_CUDA(cudaGetLastError());

    // 3. face neighbours
    m.nbr.alloc(n_t * 4);
    k_face_nbr<<<nblk(n_t * 4), 256, 0, s>>>(m.tets, n_t, m.vt_ptr, m.vt_list, m.nbr, status);
    BT_CUDA(cudaGetLastError());
    check_status(status, s, "face matching");

    // 4. CSR
    DevBuf<int32_t> row_len;
    row_len.alloc(n_dofs + 1);
    row_len.zero(s);
    k_rows<false><<<nblk(n_dofs, 128), 128, 0, s>>>(m.tets, m.comp, m.nbr, m.vt_ptr, m.vt_list, m.dof_of,
                                                    m.dof_vertex, m.dof_comp, n_dofs, nc, row_len, nullptr,
                                                    nullptr, status);
    BT_CUDA(cudaGetLastError());
    check_status(status, s, "row count");
    m.row_ptr.alloc(n_dofs + 1);
    int32_t nnz = 0;
    exclusive_scan_i32(row_len, m.row_ptr, n_dofs + 1, &nnz, s);
    m.nnz = nnz;
    m.col.alloc(nnz);
    k_rows<true><<<nblk(n_dofs, 128), 128, 0, s>>>(m.tets, m.comp, m.nbr, m.vt_ptr, m.vt_list, m.dof_of,
                                                   m.dof_vertex, m.dof_comp, n_dofs, nc, nullptr, m.row_ptr,
                                                   m.col, status);
    m.diag_pos.alloc(n_dofs);
    k_diag_pos<<<nblk(n_dofs), 256, 0, s>>>(m.row_ptr, m.col, n_dofs, m.diag_pos, status);
    BT_CUDA(cudaGetLastError());
    check_status(status, s, "row fill");

    // interface facet count (each counted from its lower-index cell)
    {
        std::vector<int32_t> hn(n_t * 4);
        m.nbr.download(hn.data(), n_t * 4, s);
        BT_CUDA(cudaStreamSynchronize(s));
        std::vector<int32_t> fc, ff;
        for (int64_t i = 0; i < n_t * 4; ++i) {
            int32_t nb = hn[i];
            int64_t t = i >> 2;
            if (nb > t && comp[nb] != comp[t]) {
                fc.push_back((int32_t)t);
                ff.push_back((int32_t)(i & 3));
            }
        }
        m.n_iface = (int64_t)fc.size();
        m.iface_cell.upload(fc.data(), fc.size(), s);
        m.iface_face.upload(ff.data(), ff.size(), s);
    }

    // 5. Jones-Plassmann colouring
    m.colour.alloc(n_t);
    BT_CUDA(cudaMemsetAsync(m.colour.p, 0xff, n_t * sizeof(int32_t), s));
    DevBuf<int32_t> selected, remaining;
    selected.alloc(n_t);
    remaining.alloc(1);
    for (int round = 0;; ++round) {
        BT_REQUIRE(round < 4096, BT_ERR_INVALID, "cell colouring did not finish");
        remaining.zero(s);
        k_jp_select<<<nblk(n_t), 256, 0, s>>>(m.tets, n_t, m.vt_ptr, m.vt_list, m.colour, selected);
        k_jp_colour<<<nblk(n_t), 256, 0, s>>>(m.tets, n_t, m.vt_ptr, m.vt_list, selected, m.colour, remaining,
                                              status);
        BT_CUDA(cudaGetLastError());
        int32_t rem = 0;
        BT_CUDA(cudaMemcpyAsync(&rem, remaining.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        BT_CUDA(cudaStreamSynchronize(s));
        if (rem == 0) break;
    }
    check_status(status, s, "colouring");
    {
        std::vector<int32_t> hc(n_t);
        m.colour.download(hc.data(), n_t, s);
        BT_CUDA(cudaStreamSynchronize(s));
        int32_t ncol = 0;
        for (int32_t c : hc) ncol = std::max(ncol, c + 1);
        std::vector<int32_t> ptr(ncol + 1, 0), cells(n_t);
        for (int32_t c : hc) ptr[c + 1]++;
        for (int c = 0; c < ncol; ++c) ptr[c + 1] += ptr[c];
        std::vector<int32_t> cur(ptr.begin(), ptr.end() - 1);
        for (int64_t t = 0; t < n_t; ++t) cells[cur[hc[t]]++] = (int32_t)t;
        m.n_colours = ncol;
        m.colour_ptr = ptr;
        m.colour_cells.upload(cells.data(), n_t, s);
    }

    // 6. sliced ELL, 32 rows per slice
    m.n_slices = (int32_t)((n_dofs + 31) / 32);
    m.sl_w.alloc(m.n_slices);
    DevBuf<int32_t> sl_entries;
    sl_entries.alloc(m.n_slices + 1);
    sl_entries.zero(s);
    k_slice_width<<<nblk(m.n_slices), 256, 0, s>>>(m.row_ptr, n_dofs, m.n_slices, m.sl_w, sl_entries);
    m.sl_ptr.alloc(m.n_slices + 1);
    int32_t sell = 0;
    exclusive_scan_i32(sl_entries, m.sl_ptr, m.n_slices + 1, &sell, s);
    m.sell_entries = sell;
    m.sl_col.alloc(sell);
    m.sl_pos.alloc(sell);
    k_slice_fill<<<nblk((int64_t)m.n_slices * 32), 256, 0, s>>>(m.row_ptr, m.col, n_dofs, m.n_slices, m.sl_ptr,
                                                               m.sl_w, m.sl_col, m.sl_pos);
    BT_CUDA(cudaGetLastError());
    BT_CUDA(cudaStreamSynchronize(s));
    m.built = true;
}

}  // namespace bt
