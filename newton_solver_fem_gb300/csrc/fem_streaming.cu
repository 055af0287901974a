// Streaming Tet4 assembly: tetrahedral topology edits (cuts that move element
// corners onto reserved copies of the original nodes) applied to fixed device
// storage.  Reference: streaming.py:1-732 (StreamingTetAssembly),
// solver.py:693-719 (prepare_tetrahedral_updates), 872-940 (refresh_topology
// with element sources).
//
// The pattern is reserved once over the candidate graph: row r holds r and
// every copy of every original neighbour of r mod N0 (N0 original nodes).
// An update then runs on the device with no host sort:
//   stage      per element: validation (source range, node range, distinct
//              original corners, every block inside the reserved pattern by a
//              binary search of the row's SELL entries) and its SELL entries;
//              nothing live changes, so a rejected update leaves the assembly
//              untouched
//   classify   the reference's lineage bookkeeping: an element keeps its
//              source's topology when its corners are unchanged (the lowest
//              such element of a source wins, deterministically), and its
//              numeric block is reusable when positions, pose and material are
//              bit-identical too; removals and topology changes mark their rows
//   publish    connectivity, poses, materials, masses and flags; contributor
//              lists rebuilt by a counting sort keyed by SELL entry (ascending
//              triplet id inside each entry) and the node incidence likewise
//   assemble   the usual deterministic gather and block-Jacobi inverse
// Reserved entries without contributors hold exact zeros, so products over the
// reserved rows equal products over the live entries.  Storage never moves,
// so a CUDA graph captured before an update replays after it.
#include <algorithm>
#include <climits>
#include <string>
#include <vector>

#include "fem_internal.cuh"

namespace fem {

namespace {

constexpr int kErrSource = 1, kErrNode = 2, kErrEdge = 3, kErrCorners = 4;
// counters: [0] error code, [1] dirty, [2] removed, [3] reused, [4] active,
// [5] touched rows, [6] topology-inserted, [7] topology-removed
constexpr int kCounters = 8;

__device__ __forceinline__ bool enabled_material(const float* mat, int e) {
    return mat[3 * e] != 0.0f || mat[3 * e + 1] != 0.0f || mat[3 * e + 2] != 0.0f;
}

__device__ __forceinline__ int corner(int4 n, int k) { return k == 0 ? n.x : (k == 1 ? n.y : (k == 2 ? n.z : n.w)); }

// SELL entry of block (row, col) by binary search of the row's columns (one
// scene: row r is lane r % 32 of slice r / 32), or -1 outside the pattern.
__device__ __forceinline__ int find_entry(int row, int col, const int* slice_ptr, const unsigned* row_info,
                                          const int* scol) {
    const int lane = row & (kSlice - 1), base = slice_ptr[row / kSlice];
    int lo = 0, hi = (int)(row_info[row] & ~kFixedBit);
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (scol[(size_t)(base + mid) * kSlice + lane] < col) lo = mid + 1;
        else hi = mid;
    }
    if (lo < (int)(row_info[row] & ~kFixedBit) && scol[(size_t)(base + lo) * kSlice + lane] == col)
        return (base + lo) * kSlice + lane;
    return -1;
}

struct StageArgs {
    int T, P, N0;
    const int4* idx;
    const float* mat;
    const int* sources;  // null: identity
    const int4* old_idx;
    const int* old_active;
    const int* slice_ptr;
    const unsigned* row_info;
    const int* scol;
    int* active;
    int* same_topo;
    int* slots;
    int* topo_winner;
    int* counters;
};

__global__ void stage_kernel(StageArgs a) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.T) return;
    a.active[e] = 0;
    a.same_topo[e] = 0;
    for (int b = 0; b < 16; ++b) a.slots[16 * e + b] = -1;
    if (!enabled_material(a.mat, e)) return;
    const int src = a.sources ? a.sources[e] : e;
    if (src < -1 || src >= a.T) {
        atomicMax(a.counters, kErrSource);
        return;
    }
    const int4 n = a.idx[e];
    for (int k = 0; k < 4; ++k) {
        const int v = corner(n, k);
        if (v < 0 || v >= a.P) {
            atomicMax(a.counters, kErrNode);
            return;
        }
        for (int j = 0; j < k; ++j)
            if (v % a.N0 == corner(n, j) % a.N0) {
                atomicMax(a.counters, kErrCorners);
                return;
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            const int entry = find_entry(corner(n, r), corner(n, c), a.slice_ptr, a.row_info, a.scol);
            if (entry < 0) {
                atomicMax(a.counters, kErrEdge);
                return;
            }
            a.slots[16 * e + 4 * r + c] = entry;
        }
    a.active[e] = 1;
    if (src >= 0 && a.old_active[src]) {
        const int4 o = a.old_idx[src];
        if (o.x == n.x && o.y == n.y && o.z == n.z && o.w == n.w) {
            a.same_topo[e] = 1;
            atomicMin(a.topo_winner + src, e);
        }
    }
}

struct ClassifyArgs {
    int T;
    const int4* idx;
    const float* pose;
    const float* mat;
    const int* sources;
    const float* old_pose;
    const float* old_mat;
    const float* q;      // current positions [3P]
    const float* lin_q;  // positions of the last linearisation [3P]
    const int* active;
    const int* same_topo;
    const int* topo_winner;
    int* reuse_src;
    int* topo_src;
    int* touched;
    int* counters;
};

__global__ void classify_kernel(ClassifyArgs a) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.T || !a.active[e]) return;
    const int src = a.sources ? a.sources[e] : e;
    const int4 n = a.idx[e];
    const bool retained = a.same_topo[e] && a.topo_winner[src] == e;
    atomicAdd(a.counters + 4, 1);
    if (!retained) {
        atomicAdd(a.counters + 6, 1);
        for (int k = 0; k < 4; ++k) a.touched[corner(n, k)] = 1;
        atomicAdd(a.counters + 1, 1);
        return;
    }
    a.topo_src[src] = 1;
    bool same = true;
    for (int k = 0; k < 4 && same; ++k)
        for (int d = 0; d < 3; ++d)
            if (a.q[3 * corner(n, k) + d] != a.lin_q[3 * corner(n, k) + d]) same = false;
    for (int k = 0; k < 3 && same; ++k)
        if (a.mat[3 * e + k] != a.old_mat[3 * src + k]) same = false;
    for (int k = 0; k < 9 && same; ++k)
        if (a.pose[9 * e + k] != a.old_pose[9 * src + k]) same = false;
    if (same) {
        a.reuse_src[src] = 1;
        atomicAdd(a.counters + 3, 1);
    } else {
        atomicAdd(a.counters + 1, 1);
    }
}

__global__ void removal_kernel(int T, const int4* __restrict__ old_idx, const int* __restrict__ old_active,
                               const int* __restrict__ reuse_src, const int* __restrict__ topo_src,
                               int* __restrict__ touched, int* __restrict__ counters) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= T || !old_active[o] || reuse_src[o]) return;
    atomicAdd(counters + 2, 1);
    if (topo_src[o]) return;
    atomicAdd(counters + 7, 1);
    const int4 n = old_idx[o];
    for (int k = 0; k < 4; ++k) touched[corner(n, k)] = 1;
}

__global__ void count_touched_kernel(int P, const int* __restrict__ touched, int* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P && touched[i]) atomicAdd(counters + 5, 1);
}

// Contributor keys: triplet t < P is row t's mass block (its diagonal entry);
// t = P + 16 e + b is block b of active tet e.
__global__ void contrib_count_kernel(int P, int T, const int* __restrict__ diag_entry, const int* __restrict__ active,
                                     const int* __restrict__ slots, int* __restrict__ count) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P) {
        atomicAdd(count + diag_entry[t], 1);
    } else if (t < P + 16 * (int64_t)T) {
        const int64_t k = t - P;
        if (active[k >> 4]) atomicAdd(count + slots[k], 1);
    }
}

__global__ void contrib_scatter_kernel(int P, int T, const int* __restrict__ diag_entry,
                                       const int* __restrict__ active, const int* __restrict__ slots,
                                       const int* __restrict__ start, int* __restrict__ count,
                                       int* __restrict__ contrib) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int entry = -1;
    if (t < P) {
        entry = diag_entry[t];
    } else if (t < P + 16 * (int64_t)T) {
        const int64_t k = t - P;
        if (active[k >> 4]) entry = slots[k];
    }
    if (entry < 0) return;
    const int pos = atomicSub(count + entry, 1) - 1;
    contrib[start[entry] + pos] = (int)t;
}

// Ascending order inside each segment [start[i], start[i+1]) (insertion sort; segments are short).
__global__ void sort_segments_kernel(int64_t n, const int* __restrict__ start, int* __restrict__ items) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int lo = start[i], hi = start[i + 1];
    for (int k = lo + 1; k < hi; ++k) {
        const int key = items[k];
        int j = k - 1;
        while (j >= lo && items[j] > key) {
            items[j + 1] = items[j];
            --j;
        }
        items[j + 1] = key;
    }
}

// Incidence over the corners of active elements only: inactive slots need not
// hold valid node indices, and their force slots are zero.
__global__ void incidence_count_kernel(int T, const int* __restrict__ idx, const int* __restrict__ active,
                                       int* __restrict__ count) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < 4 * (int64_t)T && active[k >> 2]) atomicAdd(count + idx[k], 1);
}

__global__ void incidence_scatter_kernel(int T, const int* __restrict__ idx, const int* __restrict__ active,
                                         const int* __restrict__ start, int* __restrict__ count,
                                         int* __restrict__ ent) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 4 * (int64_t)T || !active[k >> 2]) return;
    const int n = idx[k];
    const int pos = atomicSub(count + n, 1) - 1;
    ent[start[n] + pos] = (int)k;
}

// Export rows/columns of the Tet4 triplet region: the corner nodes, or -1 for an inactive element.
__global__ void tet_triplet_rc_kernel(int T, int64_t off, const int4* __restrict__ idx, const int* __restrict__ active,
                                      int* __restrict__ rows, int* __restrict__ cols) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 16 * (int64_t)T) return;
    const int e = (int)(k >> 4), b = (int)(k & 15);
    const int4 n = idx[e];
    rows[off + k] = active[e] ? corner(n, b >> 2) : -1;
    cols[off + k] = active[e] ? corner(n, b & 3) : -1;
}

const char* stage_message(int code) {
    switch (code) {
        case kErrSource: return "Element source is outside the previous element capacity";
        case kErrNode: return "Tetrahedral node is outside the reserved particle pool";
        case kErrEdge: return "Cut introduces an edge outside the reserved original-node adjacency";
        case kErrCorners: return "A tetrahedron must have four distinct original basis nodes";
        default: return "Invalid sparse topology update";
    }
}

template <class T>
cudaError_t grab(Handle& h, T** p, size_t n) {
    void* raw = nullptr;
    cudaError_t e = cudaMalloc(&raw, std::max<size_t>(1, n) * sizeof(T));
    if (e == cudaSuccess) h.allocations.push_back(raw);
    *p = static_cast<T*>(raw);
    return e;
}

}  // namespace

// Candidate pattern (streaming.py:392-420): row r holds r and every copy of
// every original neighbour of r mod N0 over the enabled tets.
int streaming_candidate(const FemDesc* d, int N0, std::vector<std::vector<int>>& rows, std::string& why) {
    const int P = d->particle_count, T = d->tet_count, copies = P / N0;
    std::vector<std::vector<int>> adj(N0);
    for (int e = 0; e < T; ++e) {
        const float* m = d->tet_materials + 3 * e;
        if (m[0] == 0.0f && m[1] == 0.0f && m[2] == 0.0f) continue;
        int o[4];
        for (int k = 0; k < 4; ++k) {
            const int v = d->tet_indices[4 * e + k];
            if (v < 0 || v >= P) {
                why = "Tetrahedral node indices are outside the reserved particle pool";
                return FEM_ERR_BAD_ARG;
            }
            o[k] = v % N0;
        }
        for (int k = 0; k < 4; ++k)
            for (int j = 0; j < k; ++j)
                if (o[k] == o[j]) {
                    why = "Each tetrahedron must have four distinct original basis nodes";
                    return FEM_ERR_BAD_ARG;
                }
        for (int k = 0; k < 4; ++k)
            for (int j = 0; j < 4; ++j)
                if (j != k) adj[o[k]].push_back(o[j]);
    }
    for (auto& a : adj) {
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
    }
    rows.assign(P, {});
    for (int r = 0; r < P; ++r) {
        std::vector<int>& c = rows[r];
        c.push_back(r);
        for (int copy = 0; copy < copies; ++copy)
            for (int n : adj[r % N0]) c.push_back(n + copy * N0);
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
    }
    return FEM_OK;
}

// Streaming buffers of a freshly built candidate-pattern handle.
cudaError_t streaming_allocate(Handle& h, int N0, const std::vector<int>& diag_entry) {
    const int T = h.T, P = h.P;
    h.orig_nodes = N0;
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
    ok(grab(h, &h.st_idx, T));
    ok(grab(h, &h.st_pose, 9 * (size_t)T));
    ok(grab(h, &h.st_mat, 3 * (size_t)T));
    ok(grab(h, &h.old_idx, T));
    ok(grab(h, &h.old_pose, 9 * (size_t)T));
    ok(grab(h, &h.old_mat, 3 * (size_t)T));
    ok(grab(h, &h.old_active, T));
    ok(grab(h, &h.lin_q, 3 * (size_t)P));
    ok(grab(h, &h.st_active, T));
    ok(grab(h, &h.st_same, T));
    ok(grab(h, &h.st_slot, 16 * (size_t)T));
    ok(grab(h, &h.topo_winner, T));
    ok(grab(h, &h.reuse_src, T));
    ok(grab(h, &h.topo_src, T));
    ok(grab(h, &h.touched, P));
    ok(grab(h, &h.counters, kCounters));
    ok(grab(h, &h.entry_count, (size_t)h.nsell));
    ok(grab(h, &h.node_count, P));
    ok(grab(h, &h.diag_entry, P));
    const int64_t scan_n = std::max<int64_t>(h.nsell, P);
    ok(grab(h, &h.scan_part, (size_t)scan_partial_count(scan_n)));
    // contributor and incidence lists at their full capacity
    ok(grab(h, &h.sell_contrib, (size_t)P + 16 * (size_t)T));
    ok(grab(h, &h.node_elem_ent, 4 * (size_t)T));
    if (e != cudaSuccess) return e;
    ok(cudaMemcpy(h.diag_entry, diag_entry.data(), sizeof(int) * (size_t)P, cudaMemcpyHostToDevice));
    ok(cudaMemset(h.old_active, 0, sizeof(int) * (size_t)T));
    ok(cudaMemset(h.entry_count, 0, sizeof(int) * (size_t)h.nsell));
    ok(cudaMemset(h.node_count, 0, sizeof(int) * (size_t)P));
    if (e == cudaSuccess) h.streaming = 1;
    return e;
}

// One topology update (streaming.py:549-700).  The new arrays come from d
// (host); q is the device positions [3P]; sources the device element lineage
// [T] or null.  Returns the lineage counters.
int streaming_update(Handle& h, const FemDesc* d, const float* q, const int* sources, FemTopologyUpdate* out,
                     cudaStream_t s, std::string& why) {
    const int T = h.T, P = h.P;
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
    // stage the new element data; the live arrays stay untouched until validation passes
    ok(cudaMemcpyAsync(h.st_idx, d->tet_indices, sizeof(int4) * (size_t)T, cudaMemcpyHostToDevice, s));
    ok(cudaMemcpyAsync(h.st_pose, d->tet_poses, sizeof(float) * 9 * (size_t)T, cudaMemcpyHostToDevice, s));
    ok(cudaMemcpyAsync(h.st_mat, d->tet_materials, sizeof(float) * 3 * (size_t)T, cudaMemcpyHostToDevice, s));
    ok(cudaMemsetAsync(h.counters, 0, sizeof(int) * kCounters, s));
    ok(cudaMemsetAsync(h.topo_winner, 0x7f, sizeof(int) * (size_t)T, s));
    ok(cudaMemsetAsync(h.reuse_src, 0, sizeof(int) * (size_t)T, s));
    ok(cudaMemsetAsync(h.topo_src, 0, sizeof(int) * (size_t)T, s));
    ok(cudaMemsetAsync(h.touched, 0, sizeof(int) * (size_t)P, s));
    if (e != cudaSuccess) return report_cuda(e);
    StageArgs sa;
    sa.T = T;
    sa.P = P;
    sa.N0 = h.orig_nodes;
    sa.idx = h.st_idx;
    sa.mat = h.st_mat;
    sa.sources = sources;
    sa.old_idx = h.old_idx;
    sa.old_active = h.old_active;
    sa.slice_ptr = h.slice_ptr;
    sa.row_info = h.row_info;
    sa.scol = h.scol;
    sa.active = h.st_active;
    sa.same_topo = h.st_same;
    sa.slots = h.st_slot;
    sa.topo_winner = h.topo_winner;
    sa.counters = h.counters;
    stage_kernel<<<blocks_for(T, 128), 128, 0, s>>>(sa);
    int code = 0;
    ok(cudaGetLastError());
    ok(cudaMemcpyAsync(&code, h.counters, sizeof(int), cudaMemcpyDeviceToHost, s));
    ok(cudaStreamSynchronize(s));
    if (e != cudaSuccess) return report_cuda(e);
    if (code != 0) {
        why = stage_message(code);
        return FEM_ERR_BAD_ARG;
    }
    ClassifyArgs ca;
    ca.T = T;
    ca.idx = h.st_idx;
    ca.pose = h.st_pose;
    ca.mat = h.st_mat;
    ca.sources = sources;
    ca.old_pose = h.old_pose;
    ca.old_mat = h.old_mat;
    ca.q = q;
    ca.lin_q = h.lin_q;
    ca.active = h.st_active;
    ca.same_topo = h.st_same;
    ca.topo_winner = h.topo_winner;
    ca.reuse_src = h.reuse_src;
    ca.topo_src = h.topo_src;
    ca.touched = h.touched;
    ca.counters = h.counters;
    classify_kernel<<<blocks_for(T, 128), 128, 0, s>>>(ca);
    removal_kernel<<<blocks_for(T, 128), 128, 0, s>>>(T, h.old_idx, h.old_active, h.reuse_src, h.topo_src, h.touched,
                                                      h.counters);
    count_touched_kernel<<<blocks_for(P, 256), 256, 0, s>>>(P, h.touched, h.counters);
    ok(cudaGetLastError());
    // publish the element, mass and flag data into the live arrays
    ok(cudaMemcpyAsync(h.tet_idx, h.st_idx, sizeof(int4) * (size_t)T, cudaMemcpyDeviceToDevice, s));
    ok(cudaMemcpyAsync(h.tet_pose, h.st_pose, sizeof(float) * 9 * (size_t)T, cudaMemcpyDeviceToDevice, s));
    ok(cudaMemcpyAsync(h.tet_mat, h.st_mat, sizeof(float) * 3 * (size_t)T, cudaMemcpyDeviceToDevice, s));
    ok(cudaMemcpyAsync(h.mass, d->particle_mass, sizeof(float) * (size_t)P, cudaMemcpyHostToDevice, s));
    ok(cudaMemcpyAsync(h.inv_mass, d->particle_inv_mass, sizeof(float) * (size_t)P, cudaMemcpyHostToDevice, s));
    if (d->particle_flags)
        ok(cudaMemcpyAsync(h.flags, d->particle_flags, sizeof(int) * (size_t)P, cudaMemcpyHostToDevice, s));
    // contributor lists keyed by SELL entry
    const int64_t nkeys = (int64_t)P + 16 * (int64_t)T;
    contrib_count_kernel<<<blocks_for(nkeys, 256), 256, 0, s>>>(P, T, h.diag_entry, h.st_active, h.st_slot,
                                                               h.entry_count);
    ok(cudaGetLastError());
    ok(launch_exclusive_scan(h.entry_count, h.sell_cptr, (int)h.nsell, h.scan_part, s));
    contrib_scatter_kernel<<<blocks_for(nkeys, 256), 256, 0, s>>>(P, T, h.diag_entry, h.st_active, h.st_slot,
                                                                 h.sell_cptr, h.entry_count, h.sell_contrib);
    sort_segments_kernel<<<blocks_for(h.nsell, 256), 256, 0, s>>>(h.nsell, h.sell_cptr, h.sell_contrib);
    // node incidence of the element-force gather (every corner slot, ascending)
    const int* flat_idx = reinterpret_cast<const int*>(h.tet_idx);
    incidence_count_kernel<<<blocks_for(4 * (int64_t)T, 256), 256, 0, s>>>(T, flat_idx, h.st_active, h.node_count);
    ok(cudaGetLastError());
    ok(launch_exclusive_scan(h.node_count, h.node_elem_ptr, P, h.scan_part, s));
    incidence_scatter_kernel<<<blocks_for(4 * (int64_t)T, 256), 256, 0, s>>>(T, flat_idx, h.st_active,
                                                                             h.node_elem_ptr, h.node_count,
                                                                             h.node_elem_ent);
    sort_segments_kernel<<<blocks_for(P, 256), 256, 0, s>>>(P, h.node_elem_ptr, h.node_elem_ent);
    tet_triplet_rc_kernel<<<blocks_for(16 * (int64_t)T, 256), 256, 0, s>>>(T, tet_triplet_offset(h), h.tet_idx,
                                                                          h.st_active, h.trip_rows, h.trip_cols);
    ok(cudaGetLastError());
    // lineage state for the next update
    ok(cudaMemcpyAsync(h.old_idx, h.st_idx, sizeof(int4) * (size_t)T, cudaMemcpyDeviceToDevice, s));
    ok(cudaMemcpyAsync(h.old_pose, h.st_pose, sizeof(float) * 9 * (size_t)T, cudaMemcpyDeviceToDevice, s));
    ok(cudaMemcpyAsync(h.old_mat, h.st_mat, sizeof(float) * 3 * (size_t)T, cudaMemcpyDeviceToDevice, s));
    ok(cudaMemcpyAsync(h.old_active, h.st_active, sizeof(int) * (size_t)T, cudaMemcpyDeviceToDevice, s));
    // numeric assembly at q (mass blocks, tangent, gather + inverse), then a cleared warm start
    ok(launch_constant_blocks(h, h.dt, s));
    ok(launch_node_prepare(h, const_cast<float*>(q), nullptr, false, false, false, s));
    ok(launch_element_tangent(h, h.dt, s));
    ok(launch_gather(h, s));
    ok(cudaMemcpyAsync(h.lin_q, q, sizeof(float) * 3 * (size_t)P, cudaMemcpyDeviceToDevice, s));
    ok(cudaMemsetAsync(h.dv, 0, sizeof(float) * 3 * (size_t)P, s));
    int c[kCounters] = {};
    ok(cudaMemcpyAsync(c, h.counters, sizeof(c), cudaMemcpyDeviceToHost, s));
    ok(cudaStreamSynchronize(s));
    if (e != cudaSuccess) return report_cuda(e);
    if (out) {
        out->dirty_elements = c[1];
        out->removed_elements = c[2];
        out->reused_elements = c[3];
        out->active_elements = c[4];
        out->touched_rows = c[5];
        out->topology_inserted_elements = c[6];
        out->topology_removed_elements = c[7];
        out->full_numeric_refresh = c[1] > c[4] / 2 ? 1 : 0;
    }
    return FEM_OK;
}

}  // namespace fem
