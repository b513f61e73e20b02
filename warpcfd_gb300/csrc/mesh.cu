// The mesh pass on the device: cells -> unique faces, owner / neighbour and the per-slot
// geometry of warp_cfd/preprocess/mesh.py:64-302, for meshes of millions of cells (the host
// pass sorts 12.6M face rows of a 2.1M-cell hex mesh in numpy for ~15 s).
//
// Face matching without a general sort.  Every (cell, face) entry of one node count (the
// triangle set, then the quad set, numbered in that order as the reference numbers a wedge
// mesh's faces) gets its key = the face's node ids sorted ascending.  Faces are numbered in
// lexicographic order of their keys (np.unique(axis=0) at mesh.py:121), and the first key
// component is a node id, so a counting sort on it -- a histogram over the nodes, an
// exclusive scan, a scatter -- puts the entries into per-node buckets that are already in
// face-number order; each bucket holds a handful of entries (at most 12 in a hex lattice)
// and one thread sorts it by (rest of key, entry index) and counts its distinct keys.  A
// second scan of those counts gives every bucket its first face id; the emitting pass then
// writes the unique faces and, per face, the owner (the lower cell: entries of a key are in
// entry = cell-major order) and the neighbour.  Bit-identical topology to the host pass.
//
// Geometry in float64 with the host pass's order of operations and no contraction
// (__dmul_rn / __dadd_rn / __dsub_rn): the fan triangulation of mesh.py:161-183 as numpy
// evaluates np.cross and np.linalg.norm, node means summed in index order.  The cell volume
// (an einsum on the host) is summed here slot by slot.
#include <climits>
#include <cstdint>
#include <cstdio>

#include "common.cuh"

namespace {

thread_local char g_mesh_error[256] = "";

constexpr int kKinds = 3;       // 0 hexahedron, 1 wedge, 2 tetrahedron
constexpr int kScanItems = 4;   // elements per thread in the scan
constexpr int kScanBlock = 1024;

struct FaceTable {
    int nf;            // faces of the cell type
    int npf[6];        // nodes of each face
    int node[6][4];    // local node ids of each face, in the cell's own order
};

// local face -> local node tables of mesh.py:69-91 (the wedge's triangles first)
__constant__ FaceTable c_tables[kKinds] = {
    {6, {4, 4, 4, 4, 4, 4}, {{3, 2, 1, 0}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {3, 7, 6, 2}, {3, 0, 4, 7}}},
    {5, {3, 3, 4, 4, 4, 0}, {{0, 2, 1, 0}, {3, 4, 5, 0}, {0, 3, 5, 2}, {1, 2, 5, 4}, {0, 1, 4, 3}, {0, 0, 0, 0}}},
    {4, {3, 3, 3, 3, 0, 0}, {{2, 1, 0, 0}, {0, 1, 3, 0}, {3, 2, 0, 0}, {1, 2, 3, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}}},
};

__device__ __forceinline__ int kind_of(int vtk) {
    return vtk == 12 ? 0 : vtk == 13 ? 1 : vtk == 10 ? 2 : -1;
}

__device__ __forceinline__ int nodes_of_kind(int k) { return k == 0 ? 8 : k == 1 ? 6 : 4; }

// slot of the j-th face with `npf` nodes of a cell of kind k, or -1
__device__ __forceinline__ int set_slot(int k, int npf, int j) {
    const FaceTable& t = c_tables[k];
    int seen = 0;
    for (int f = 0; f < t.nf; ++f) {
        if (t.npf[f] == npf) {
            if (seen == j) return f;
            ++seen;
        }
    }
    return -1;
}

// error bits
constexpr int kErrNode = 1;       // node id out of range
constexpr int kErrShared = 2;     // a face shared by more than two cells
constexpr int kErrSelf = 4;       // a cell sharing a face with itself
constexpr int kErrType = 8;       // unsupported cell type
constexpr int kErrSlots = 16;     // a cell with more faces than faces_per_cell / the set's slots

__device__ __forceinline__ void cswap(int& a, int& b) {
    const int lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

__global__ void face_keys_kernel(const int32_t* __restrict__ cells, const int32_t* __restrict__ type, int C,
                                 int P, int F, int npf, int S, int4* __restrict__ keys, int* __restrict__ count,
                                 int* __restrict__ err) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)C * S) return;
    const int c = (int)(e / S), j = (int)(e % S);
    const int k = kind_of(type[c]);
    int4 key = make_int4(-1, -1, -1, -1);
    if (k < 0) {
        atomicOr(err, kErrType);
    } else if (c_tables[k].nf > F || set_slot(k, npf, S) >= 0) {
        atomicOr(err, kErrSlots);  // the slot table cannot hold this cell's faces
    } else {
        const int slot = set_slot(k, npf, j);
        if (slot >= 0) {
            int v[4];
            bool ok = true;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                v[i] = i < npf ? cells[8 * (size_t)c + c_tables[k].node[slot][i]] : INT_MAX;
                if (i < npf && (v[i] < 0 || v[i] >= P)) ok = false;
            }
            if (!ok) {
                atomicOr(err, kErrNode);
            } else {
                cswap(v[0], v[1]);
                cswap(v[2], v[3]);
                cswap(v[0], v[2]);
                cswap(v[1], v[3]);
                cswap(v[1], v[2]);
                key = make_int4(v[0], v[1], v[2], npf == 4 ? v[3] : -1);
                atomicAdd(count + v[0], 1);
            }
        }
    }
    keys[e] = key;
}

// In-place exclusive scan of n ints in three kernels: per-block scans (kScanItems per
// thread) with the block totals to `sums`, one block scanning `sums`, then the offsets.
__device__ __forceinline__ int block_exclusive_scan(int v, int* s_warp, int* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        s_warp[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    const int before = (w > 0 ? s_warp[w - 1] : 0) + x - v;
    *total = s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(kScanBlock) scan_blocks_kernel(int* __restrict__ a, long long n, int* __restrict__ sums) {
    __shared__ int s_warp[32];
    const long long base = (long long)blockIdx.x * kScanBlock * kScanItems + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int t = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? a[base + i] : 0;
        t += v[i];
    }
    int total;
    int run = block_exclusive_scan(t, s_warp, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) a[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) scan_sums_kernel(int* __restrict__ sums, int nb, int* __restrict__ total_out) {
    __shared__ int s_warp[32];
    int carry = 0;
    for (int base = 0; base < nb; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, s_warp, &total);
        if (i < nb) sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void __launch_bounds__(kScanBlock) scan_add_kernel(int* __restrict__ a, long long n, const int* __restrict__ sums) {
    const long long base = (long long)blockIdx.x * kScanBlock * kScanItems + (long long)threadIdx.x * kScanItems;
    const int off = sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) a[base + i] += off;
}

__global__ void scatter_kernel(const int4* __restrict__ keys, long long E, const int* __restrict__ start,
                               int* __restrict__ fill, int* __restrict__ perm) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int b = keys[e].x;
    if (b < 0) return;
    perm[start[b] + atomicAdd(fill + b, 1)] = (int)e;
}

__device__ __forceinline__ bool same_key(const int4& a, const int4& b) {
    return a.y == b.y && a.z == b.z && a.w == b.w;  // x equal inside a bucket
}

__device__ __forceinline__ bool key_less(const int4& a, int ea, const int4& b, int eb) {
    if (a.y != b.y) return a.y < b.y;
    if (a.z != b.z) return a.z < b.z;
    if (a.w != b.w) return a.w < b.w;
    return ea < eb;
}

// one thread per node bucket: insertion sort by (key, entry), distinct keys -> ucount
__global__ void bucket_sort_kernel(const int4* __restrict__ keys, const int* __restrict__ start, int P, int S,
                                   int* __restrict__ perm, int* __restrict__ ucount, int* __restrict__ err) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P) return;
    const int s = start[b], n = start[b + 1] - s;
    int* q = perm + s;
    for (int i = 1; i < n; ++i) {
        const int e = q[i];
        const int4 ke = keys[e];
        int j = i - 1;
        while (j >= 0 && key_less(ke, e, keys[q[j]], q[j])) {
            q[j + 1] = q[j];
            --j;
        }
        q[j + 1] = e;
    }
    int u = 0, run = 0;
    int4 prev = make_int4(0, 0, 0, 0);
    int prev_cell = -1;
    for (int i = 0; i < n; ++i) {
        const int e = q[i];
        const int4 k = keys[e];
        const int cell = e / S;
        if (i == 0 || !same_key(k, prev)) {
            ++u;
            run = 1;
        } else {
            ++run;
            if (run > 2) atomicOr(err, kErrShared);
            if (cell == prev_cell) atomicOr(err, kErrSelf);
        }
        prev = k;
        prev_cell = cell;
    }
    ucount[b] = u;
}

struct EmitArgs {
    const int4* keys;
    const int* start;
    const int* fbase;
    const int* perm;
    const int32_t* type;
    int P, S, npf, F, shift, width;
    int32_t* cell_faces;
    int32_t* unique_faces;
    int32_t* face_nodes;
    int32_t* face_cells;
    int32_t* face_slots;
};

__global__ void emit_kernel(EmitArgs a) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= a.P) return;
    const int s = a.start[b], n = a.start[b + 1] - s;
    int id = a.shift + a.fbase[b] - 1;
    int4 prev = make_int4(0, 0, 0, 0);
    for (int i = 0; i < n; ++i) {
        const int e = a.perm[s + i];
        const int4 k = a.keys[e];
        const int c = e / a.S, j = e % a.S;
        const int slot = set_slot(kind_of(a.type[c]), a.npf, j);
        if (i == 0 || !same_key(k, prev)) {
            ++id;
            int32_t* row = a.unique_faces + (size_t)id * a.width;
            row[0] = k.x;
            row[1] = k.y;
            row[2] = k.z;
            if (a.width > 3) row[3] = a.npf == 4 ? k.w : -1;
            a.face_nodes[id] = a.npf;
            a.face_cells[2 * (size_t)id] = c;
            a.face_slots[2 * (size_t)id] = slot;
            a.face_cells[2 * (size_t)id + 1] = -1;
            a.face_slots[2 * (size_t)id + 1] = -1;
        } else {
            a.face_cells[2 * (size_t)id + 1] = c;
            a.face_slots[2 * (size_t)id + 1] = slot;
        }
        a.cell_faces[(size_t)c * a.F + slot] = id;
        prev = k;
    }
}

struct Vec3 {
    double x, y, z;
};

__device__ __forceinline__ Vec3 ld_point(const double* p, int i) {
    return {p[3 * (size_t)i], p[3 * (size_t)i + 1], p[3 * (size_t)i + 2]};
}
__device__ __forceinline__ Vec3 vsub(Vec3 a, Vec3 b) {
    return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)};
}
__device__ __forceinline__ Vec3 vadd(Vec3 a, Vec3 b) {
    return {__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)};
}

// cell centre = node mean (VTK's parametric centre of a linear cell), nodes summed in order
__global__ void cell_centroid_kernel(const double* __restrict__ pts, const int32_t* __restrict__ cells,
                                     const int32_t* __restrict__ type, int C, double* __restrict__ cent) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const int k = kind_of(type[c]);
    if (k < 0) return;
    const int nn = nodes_of_kind(k);
    Vec3 s = ld_point(pts, cells[8 * (size_t)c]);
    for (int i = 1; i < nn; ++i) s = vadd(s, ld_point(pts, cells[8 * (size_t)c + i]));
    const double d = (double)nn;
    cent[3 * (size_t)c] = __ddiv_rn(s.x, d);
    cent[3 * (size_t)c + 1] = __ddiv_rn(s.y, d);
    cent[3 * (size_t)c + 2] = __ddiv_rn(s.z, d);
}

// face centroid = mean of its (sorted) nodes
__global__ void face_centroid_kernel(const double* __restrict__ pts, const int32_t* __restrict__ unique_faces,
                                     const int32_t* __restrict__ face_nodes, int K, int width,
                                     double* __restrict__ fc) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= K) return;
    const int n = face_nodes[f];
    const int32_t* row = unique_faces + (size_t)f * width;
    Vec3 s = ld_point(pts, row[0]);
    for (int i = 1; i < n; ++i) s = vadd(s, ld_point(pts, row[i]));
    const double d = (double)n;
    fc[3 * (size_t)f] = __ddiv_rn(s.x, d);
    fc[3 * (size_t)f + 1] = __ddiv_rn(s.y, d);
    fc[3 * (size_t)f + 2] = __ddiv_rn(s.z, d);
}

// per (cell, slot): fan-triangulated area and unit normal from the cell's own node order
// (mesh.py:161-183), centroid -> face-centroid vector; zeros on null slots
__global__ void slot_geometry_kernel(const double* __restrict__ pts, const int32_t* __restrict__ cells,
                                     const int32_t* __restrict__ type, const int32_t* __restrict__ cell_faces,
                                     const double* __restrict__ cent, const double* __restrict__ fc, int C, int F,
                                     double* __restrict__ area, double* __restrict__ normal,
                                     double* __restrict__ to_face) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)C * F) return;
    const int c = (int)(t / F), slot = (int)(t % F);
    const int k = kind_of(type[c]);
    const int fid = cell_faces[t];
    if (k < 0 || slot >= c_tables[k].nf || fid < 0) {
        area[t] = 0.0;
        normal[3 * t] = normal[3 * t + 1] = normal[3 * t + 2] = 0.0;
        to_face[3 * t] = to_face[3 * t + 1] = to_face[3 * t + 2] = 0.0;
        return;
    }
    const int npf = c_tables[k].npf[slot];
    const int32_t* cn = cells + 8 * (size_t)c;
    const Vec3 v0 = ld_point(pts, cn[c_tables[k].node[slot][0]]);
    double A = 0.0;
    Vec3 vec = {0.0, 0.0, 0.0};
    for (int i = 1; i < npf - 1; ++i) {
        const Vec3 a = vsub(ld_point(pts, cn[c_tables[k].node[slot][i]]), v0);
        const Vec3 b = vsub(ld_point(pts, cn[c_tables[k].node[slot][i + 1]]), v0);
        // np.cross: (a1 b2 - a2 b1, a2 b0 - a0 b2, a0 b1 - a1 b0), each product rounded
        const Vec3 cr = {__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)),
                         __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
                         __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
        const Vec3 nv = {__dmul_rn(0.5, cr.x), __dmul_rn(0.5, cr.y), __dmul_rn(0.5, cr.z)};
        const double n2 = __dadd_rn(__dadd_rn(__dmul_rn(nv.x, nv.x), __dmul_rn(nv.y, nv.y)), __dmul_rn(nv.z, nv.z));
        A = __dadd_rn(A, __dsqrt_rn(n2));
        vec = vadd(vec, nv);
    }
    area[t] = A;
    normal[3 * t] = __ddiv_rn(vec.x, A);
    normal[3 * t + 1] = __ddiv_rn(vec.y, A);
    normal[3 * t + 2] = __ddiv_rn(vec.z, A);
    to_face[3 * t] = __dsub_rn(fc[3 * (size_t)fid], cent[3 * (size_t)c]);
    to_face[3 * t + 1] = __dsub_rn(fc[3 * (size_t)fid + 1], cent[3 * (size_t)c + 1]);
    to_face[3 * t + 2] = __dsub_rn(fc[3 * (size_t)fid + 2], cent[3 * (size_t)c + 2]);
}

// |sum over slots of (n A) . r_f| / 3, the divergence theorem over the fan-triangulated faces
__global__ void volume_kernel(const double* __restrict__ area, const double* __restrict__ normal,
                              const int32_t* __restrict__ cell_faces, const double* __restrict__ fc, int C, int F,
                              double* __restrict__ vol) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double s = 0.0;
    for (int f = 0; f < F; ++f) {
        const size_t t = (size_t)c * F + f;
        const int fid = cell_faces[t];
        if (fid < 0) continue;
        const double A = area[t];
        s = __dadd_rn(s, __dmul_rn(__dmul_rn(normal[3 * t], A), fc[3 * (size_t)fid]));
        s = __dadd_rn(s, __dmul_rn(__dmul_rn(normal[3 * t + 1], A), fc[3 * (size_t)fid + 1]));
        s = __dadd_rn(s, __dmul_rn(__dmul_rn(normal[3 * t + 2], A), fc[3 * (size_t)fid + 2]));
    }
    vol[c] = fabs(__ddiv_rn(s, 3.0));
}

// ---------------------------------------------------------------- workspace layout
struct SetLayout {
    size_t keys, perm, start, fill, fbase;  // byte offsets
    int S;
};

struct Layout {
    SetLayout set[2];  // triangles, quads
    size_t sums, scalars, bytes;
    int nb_nodes;      // scan blocks over P + 1 entries
};

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

Layout layout_of(const wcfd_mesh_cells* m) {
    Layout L{};
    size_t off = 0;
    const long long P1 = (long long)m->n_points + 1;
    for (int s = 0; s < 2; ++s) {
        SetLayout& q = L.set[s];
        q.S = s == 0 ? m->tri_slots : m->quad_slots;
        const size_t E = (size_t)m->n_cells * (size_t)q.S;
        q.keys = off;  off = align16(off + E * sizeof(int4));
        q.perm = off;  off = align16(off + E * sizeof(int));
        q.start = off; off = align16(off + P1 * sizeof(int));
        q.fill = off;  off = align16(off + P1 * sizeof(int));
        q.fbase = off; off = align16(off + P1 * sizeof(int));
    }
    L.nb_nodes = (int)((P1 + (long long)kScanBlock * kScanItems - 1) / ((long long)kScanBlock * kScanItems));
    L.sums = off;    off = align16(off + (size_t)(L.nb_nodes + 1) * sizeof(int));
    L.scalars = off; off = align16(off + 8 * sizeof(int));  // [0] error bits, [1] scan total, [2..3] faces per set
    L.bytes = off;
    return L;
}

int mesh_error(int code, const char* what) {
    std::snprintf(g_mesh_error, sizeof(g_mesh_error), "%s", what);
    return code;
}

int check_cells(const wcfd_mesh_cells* m) {
    if (!m || !m->points || !m->cells || !m->cell_type) return mesh_error(WCFD_ERR_ARGUMENT, "null mesh cells");
    if (m->n_cells <= 0 || m->n_points <= 0) return mesh_error(WCFD_ERR_ARGUMENT, "empty mesh");
    if (m->faces_per_cell < 4 || m->faces_per_cell > wcfd::kMaxSlots || m->tri_slots < 0 || m->tri_slots > 4 ||
        m->quad_slots < 0 || m->quad_slots > 6 || (m->tri_slots == 0 && m->quad_slots == 0))
        return mesh_error(WCFD_ERR_ARGUMENT, "bad faces_per_cell / tri_slots / quad_slots");
    if ((long long)m->n_cells * 6 >= INT_MAX) return mesh_error(WCFD_ERR_TOO_LARGE, "more than 357M cells");
    return WCFD_OK;
}

#define MESH_CHECK(what)                                                                          \
    do {                                                                                          \
        const cudaError_t e_ = cudaGetLastError();                                                \
        if (e_ != cudaSuccess) {                                                                  \
            std::snprintf(g_mesh_error, sizeof(g_mesh_error), "%s: %s", what, cudaGetErrorString(e_)); \
            return WCFD_ERR_CUDA;                                                                 \
        }                                                                                         \
    } while (0)

int exclusive_scan(int* a, long long n, int* sums, int* total, cudaStream_t st) {
    const int nb = (int)((n + (long long)kScanBlock * kScanItems - 1) / ((long long)kScanBlock * kScanItems));
    scan_blocks_kernel<<<nb, kScanBlock, 0, st>>>(a, n, sums);
    scan_sums_kernel<<<1, kScanBlock, 0, st>>>(sums, nb, total);
    scan_add_kernel<<<nb, kScanBlock, 0, st>>>(a, n, sums);
    MESH_CHECK("scan");
    return WCFD_OK;
}

int blocks_for(long long n, int bs) { return (int)((n + bs - 1) / bs); }

// Validation of a device geometry (the index arrays every kernel gathers through): each
// check reads an index only after the bounds it is used under have been checked, and each
// violation adds one to a counter per kind.
//   [0] face owner outside [0, C) or neighbour outside [-1, C) or equal to the owner
//   [1] boundary row of a boundary face outside [0, B)
//   [2] a cell slot that is not null and names a face outside [0, K)
//   [3] a cell slot whose face does not have this cell on the side the slot says
//   [4] an off-diagonal column outside [0, C), or (with ell_dcol) an offset that does not
//       give the column
constexpr int kChecks = 5;

__global__ void check_faces_kernel(wcfd_mesh m, int* __restrict__ bad) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_faces) return;
    const int P = m.face_owner[k], N = m.face_nbr[k];
    if (P < 0 || P >= m.n_cells || N < -1 || N >= m.n_cells || N == P) atomicAdd(bad + 0, 1);
    if (N < 0) {
        const int b = m.face_brow[k];
        if (b < 0 || b >= m.n_bfaces) atomicAdd(bad + 1, 1);
    }
}

__global__ void check_cells_kernel(wcfd_mesh m, int* __restrict__ bad) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    const float4* slots = reinterpret_cast<const float4*>(m.cell_slot);
    for (int f = 0; f < m.faces_per_cell; ++f) {
        const int sk = __float_as_int(slots[(size_t)f * m.n_cells + c].w);
        if (sk == wcfd::kNullSlot) continue;
        const int k = sk >= 0 ? sk : ~sk;
        if (k < 0 || k >= m.n_faces) {
            atomicAdd(bad + 2, 1);
            continue;
        }
        if ((sk >= 0 ? m.face_owner[k] : m.face_nbr[k]) != c) atomicAdd(bad + 3, 1);
    }
    for (int j = 0; j < m.ell_width; ++j) {
        const int col = m.ell_col[(size_t)j * m.n_cells + c];
        if (col < 0 || col >= m.n_cells) atomicAdd(bad + 4, 1);
        else if (m.ell_dcol && c + (int)m.ell_dcol[(size_t)j * m.n_cells + c] != col) atomicAdd(bad + 4, 1);
    }
}

}  // namespace

extern "C" {

const char* wcfd_mesh_last_error(void) { return g_mesh_error; }

int wcfd_check_mesh(const wcfd_mesh* m, int32_t* counts, void* stream) {
    if (!m || !counts) return mesh_error(WCFD_ERR_ARGUMENT, "null mesh or counts");
    if (m->n_cells <= 0 || m->n_faces <= 0 || m->faces_per_cell < 1 || m->faces_per_cell > wcfd::kMaxSlots ||
        m->ell_width < 0 || m->ell_width > m->faces_per_cell)
        return mesh_error(WCFD_ERR_ARGUMENT, "bad mesh sizes");
    if (!m->face_owner || !m->face_nbr || !m->face_brow || !m->cell_slot || !m->ell_col)
        return mesh_error(WCFD_ERR_ARGUMENT, "mesh has a null index array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int* bad = nullptr;
    if (cudaMalloc(&bad, kChecks * sizeof(int)) != cudaSuccess) MESH_CHECK("allocation");
    int rc = WCFD_OK;
    if (cudaMemsetAsync(bad, 0, kChecks * sizeof(int), st) != cudaSuccess) rc = WCFD_ERR_CUDA;
    if (rc == WCFD_OK) {
        check_faces_kernel<<<blocks_for(m->n_faces, 256), 256, 0, st>>>(*m, bad);
        check_cells_kernel<<<blocks_for(m->n_cells, 256), 256, 0, st>>>(*m, bad);
        int host[kChecks] = {0, 0, 0, 0, 0};
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(host, bad, sizeof(host), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = WCFD_ERR_CUDA;
        } else {
            int total = 0;
            for (int i = 0; i < kChecks; ++i) {
                counts[i] = host[i];
                total += host[i];
            }
            if (total) {
                std::snprintf(g_mesh_error, sizeof(g_mesh_error),
                              "mesh index check: %d bad face ids, %d bad boundary rows, %d bad slot faces, "
                              "%d slot/face mismatches, %d bad columns", host[0], host[1], host[2], host[3], host[4]);
                rc = WCFD_ERR_ARGUMENT;
            }
        }
    }
    if (rc == WCFD_ERR_CUDA) std::snprintf(g_mesh_error, sizeof(g_mesh_error), "mesh index check: %s",
                                           cudaGetErrorString(cudaGetLastError()));
    cudaFree(bad);
    return rc;
}

size_t wcfd_mesh_workspace_bytes(const wcfd_mesh_cells* m) {
    if (check_cells(m) != WCFD_OK) return 0;
    return layout_of(m).bytes;
}

int wcfd_mesh_match_faces(const wcfd_mesh_cells* m, void* ws, size_t ws_bytes, int32_t* n_faces, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = check_cells(m);
    if (rc != WCFD_OK) return rc;
    const Layout L = layout_of(m);
    if (!ws || ws_bytes < L.bytes || !n_faces) return mesh_error(WCFD_ERR_ARGUMENT, "workspace too small or null");
    char* base = static_cast<char*>(ws);
    int* scalars = reinterpret_cast<int*>(base + L.scalars);
    int* sums = reinterpret_cast<int*>(base + L.sums);
    const int C = m->n_cells, P = m->n_points, F = m->faces_per_cell;
    if (cudaMemsetAsync(scalars, 0, 8 * sizeof(int), st) != cudaSuccess) MESH_CHECK("memset");
    for (int s = 0; s < 2; ++s) {
        const SetLayout& q = L.set[s];
        if (q.S == 0) continue;
        const int npf = s == 0 ? 3 : 4;
        int4* keys = reinterpret_cast<int4*>(base + q.keys);
        int* perm = reinterpret_cast<int*>(base + q.perm);
        int* start = reinterpret_cast<int*>(base + q.start);
        int* fill = reinterpret_cast<int*>(base + q.fill);
        int* fbase = reinterpret_cast<int*>(base + q.fbase);
        const long long E = (long long)C * q.S;
        if (cudaMemsetAsync(start, 0, (size_t)(P + 1) * sizeof(int), st) != cudaSuccess ||
            cudaMemsetAsync(fill, 0, (size_t)(P + 1) * sizeof(int), st) != cudaSuccess)
            MESH_CHECK("memset");
        face_keys_kernel<<<blocks_for(E, 256), 256, 0, st>>>(m->cells, m->cell_type, C, P, F, npf, q.S, keys,
                                                             start, scalars);
        MESH_CHECK("face keys");
        rc = exclusive_scan(start, (long long)P + 1, sums, scalars + 1, st);
        if (rc != WCFD_OK) return rc;
        scatter_kernel<<<blocks_for(E, 256), 256, 0, st>>>(keys, E, start, fill, perm);
        MESH_CHECK("scatter");
        bucket_sort_kernel<<<blocks_for(P, 128), 128, 0, st>>>(keys, start, P, q.S, perm, fbase, scalars);
        MESH_CHECK("bucket sort");
        if (cudaMemsetAsync(fbase + P, 0, sizeof(int), st) != cudaSuccess) MESH_CHECK("memset");
        rc = exclusive_scan(fbase, (long long)P + 1, sums, scalars + 2 + s, st);
        if (rc != WCFD_OK) return rc;
    }
    int host[4] = {0, 0, 0, 0};
    if (cudaMemcpyAsync(host, scalars, sizeof(host), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        MESH_CHECK("read counts");
    if (host[0] & kErrType) return mesh_error(WCFD_ERR_ARGUMENT, "only Tetra and Hexahedron and Wedge elements are supported");
    if (host[0] & kErrSlots) return mesh_error(WCFD_ERR_ARGUMENT, "faces_per_cell / tri_slots / quad_slots too small for a cell type present");
    if (host[0] & kErrNode) return mesh_error(WCFD_ERR_ARGUMENT, "a cell references a node id out of range");
    if (host[0] & kErrShared) return mesh_error(WCFD_ERR_ARGUMENT, "a face is shared by more than two cells");
    if (host[0] & kErrSelf) return mesh_error(WCFD_ERR_ARGUMENT, "a cell shares a face with itself");
    n_faces[0] = L.set[0].S ? host[2] : 0;
    n_faces[1] = L.set[1].S ? host[3] : 0;
    return WCFD_OK;
}

int wcfd_mesh_emit(const wcfd_mesh_cells* m, void* ws, size_t ws_bytes, const int32_t* n_faces,
                   const wcfd_mesh_faces* out, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = check_cells(m);
    if (rc != WCFD_OK) return rc;
    const Layout L = layout_of(m);
    if (!ws || ws_bytes < L.bytes || !n_faces || !out) return mesh_error(WCFD_ERR_ARGUMENT, "null argument");
    if (!out->cell_faces || !out->unique_faces || !out->face_nodes || !out->face_cells || !out->face_slots ||
        !out->centroid || !out->volume || !out->area || !out->normal || !out->to_face || !out->face_centroid)
        return mesh_error(WCFD_ERR_ARGUMENT, "null output array");
    const int width = L.set[1].S ? 4 : 3;
    if (out->node_width != width) return mesh_error(WCFD_ERR_ARGUMENT, "node_width must be 4 with quads, else 3");
    char* base = static_cast<char*>(ws);
    const int C = m->n_cells, P = m->n_points, F = m->faces_per_cell;
    const int K = n_faces[0] + n_faces[1];
    if (cudaMemsetAsync(out->cell_faces, 0xff, (size_t)C * F * sizeof(int32_t), st) != cudaSuccess)
        MESH_CHECK("memset");
    int shift = 0;
    for (int s = 0; s < 2; ++s) {
        const SetLayout& q = L.set[s];
        if (q.S == 0) continue;
        EmitArgs a;
        a.keys = reinterpret_cast<const int4*>(base + q.keys);
        a.start = reinterpret_cast<const int*>(base + q.start);
        a.fbase = reinterpret_cast<const int*>(base + q.fbase);
        a.perm = reinterpret_cast<const int*>(base + q.perm);
        a.type = m->cell_type;
        a.P = P;
        a.S = q.S;
        a.npf = s == 0 ? 3 : 4;
        a.F = F;
        a.shift = shift;
        a.width = width;
        a.cell_faces = out->cell_faces;
        a.unique_faces = out->unique_faces;
        a.face_nodes = out->face_nodes;
        a.face_cells = out->face_cells;
        a.face_slots = out->face_slots;
        emit_kernel<<<blocks_for(P, 128), 128, 0, st>>>(a);
        MESH_CHECK("emit");
        shift += n_faces[s];
    }
    cell_centroid_kernel<<<blocks_for(C, 256), 256, 0, st>>>(m->points, m->cells, m->cell_type, C, out->centroid);
    face_centroid_kernel<<<blocks_for(K, 256), 256, 0, st>>>(m->points, out->unique_faces, out->face_nodes, K, width,
                                                             out->face_centroid);
    slot_geometry_kernel<<<blocks_for((long long)C * F, 256), 256, 0, st>>>(
        m->points, m->cells, m->cell_type, out->cell_faces, out->centroid, out->face_centroid, C, F, out->area,
        out->normal, out->to_face);
    volume_kernel<<<blocks_for(C, 256), 256, 0, st>>>(out->area, out->normal, out->cell_faces, out->face_centroid, C,
                                                      F, out->volume);
    MESH_CHECK("mesh geometry");
    return WCFD_OK;
}

}  // extern "C"
