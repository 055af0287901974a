// Contact force terms of the substep, deterministic (no float atomics):
//
//   particle-particle self contact (reference kernels.py:1036-1114; the hash
//   grid of solver.py:1477-1511).  The grid is rebuilt at every evaluation:
//   active particles are bucketed by cell floor(x / w), w = 2 max_radius +
//   cohesion, with cell coordinates wrapped onto grid_dim^3 buckets; bucket
//   counts are scanned, particles scattered, and every bucket sorted by
//   particle id.  Each particle then visits the cells its query sphere
//   (radius r_i + max_radius + cohesion <= w, so at most 3 cells per axis)
//   overlaps, in a fixed order, and sums the penalty + damping + Coulomb
//   force over neighbours with d - r_i - r_j <= cohesion: the reference's
//   neighbour set, summed in a fixed order instead of hash-query order.
//
//   soft-rigid contact (kernels.py:1198-1261): one thread per listed contact
//   computes the penalty + damping + capped Coulomb force of a penetrating
//   contact and links it into its particle's list; the node gather adds each
//   list in ascending contact id.
#include <climits>

#include "fem_internal.cuh"
#include "fem_math.cuh"

namespace fem {

namespace {


__device__ __forceinline__ int cell_coord(float x, float inv_w) {
    const float c = floorf(x * inv_w);
    return (int)fminf(fmaxf(c, -1.0e9f), 1.0e9f);
}

__device__ __forceinline__ int bucket_of(int cx, int cy, int cz, int dim) {
    const int m = dim - 1;  // dim is a power of two: & gives the non-negative remainder
    return ((cz & m) * dim + (cy & m)) * dim + (cx & m);
}

__global__ void grid_count_kernel(int P, const float4* __restrict__ q4, const int* __restrict__ flags, float inv_w,
                                  int dim, int* __restrict__ cell_of, int* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    if ((flags[i] & 1) == 0) {
        cell_of[i] = -1;
        return;
    }
    const float4 x = q4[i];
    const int b = bucket_of(cell_coord(x.x, inv_w), cell_coord(x.y, inv_w), cell_coord(x.z, inv_w), dim);
    cell_of[i] = b;
    atomicAdd(count + b, 1);
}

}  // namespace

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

// Exclusive scan of count[0, n) into start[0, n]: tile sums, a one-CTA scan of
// the tile sums, then each tile's scan plus its offset.
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) warp_sums[lane] = w;  // inclusive warp prefix
    }
    __syncthreads();
    total = warp_sums[(blockDim.x >> 5) - 1];
    const int before = warp == 0 ? 0 : warp_sums[warp - 1];
    __syncthreads();
    return before + incl - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_tile_sums_kernel(int n, const int* __restrict__ count,
                                                                      int* __restrict__ part) {
    __shared__ int warp_sums[32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) v += count[base + k];
    int total;
    block_exclusive_scan(v, warp_sums, total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_part_kernel(int nparts, int* __restrict__ part) {
    __shared__ int warp_sums[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nparts; b0 += kScanThreads) {
        const int k = b0 + threadIdx.x;
        const int v = k < nparts ? part[k] : 0;
        int total;
        const int ex = block_exclusive_scan(v, warp_sums, total);
        if (k < nparts) part[k] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(int n, const int* __restrict__ count,
                                                                  const int* __restrict__ part, int* __restrict__ start,
                                                                  int grand_total_slot) {
    __shared__ int warp_sums[32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int c[kScanItems];
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        c[k] = base + k < n ? count[base + k] : 0;
        v += c[k];
    }
    int total;
    int run = part[blockIdx.x] + block_exclusive_scan(v, warp_sums, total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) start[base + k] = run;
        run += c[k];
    }
    if (grand_total_slot && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) start[n] = run;
}

}  // namespace

int scan_partial_count(int64_t n) { return (int)((n + kScanTile - 1) / kScanTile); }

cudaError_t launch_exclusive_scan(const int* count, int* start, int n, int* part, cudaStream_t s) {
    if (n <= 0) return cudaMemsetAsync(start, 0, sizeof(int), s);
    const int tiles = scan_partial_count(n);
    scan_tile_sums_kernel<<<tiles, kScanThreads, 0, s>>>(n, count, part);
    scan_part_kernel<<<1, kScanThreads, 0, s>>>(tiles, part);
    scan_tiles_kernel<<<tiles, kScanThreads, 0, s>>>(n, count, part, start, 1);
    return cudaGetLastError();
}

namespace {

// Scatter: each particle takes a position in its bucket by decrementing the
// bucket count, which leaves every count at zero for the next evaluation.
__global__ void grid_scatter_kernel(int P, const int* __restrict__ cell_of, const int* __restrict__ start,
                                    int* __restrict__ count, int* __restrict__ items) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int b = cell_of[i];
    if (b < 0) return;
    const int k = atomicSub(count + b, 1) - 1;
    items[start[b] + k] = i;
}

// Sort every bucket by particle id (insertion sort; buckets are short), so the
// neighbour order no longer depends on the scatter order.
__global__ void grid_sort_kernel(int nb, const int* __restrict__ start, int* __restrict__ items) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int lo = start[b], hi = start[b + 1];
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

struct ParticleContactArgs {
    int P, dim;
    float inv_w, ke, kd, kf, mu, cohesion, max_radius;
    const float4* q4;
    const float4* v4;
    const float* radius;
    const int* flags;
    const int* start;
    const int* items;
    float4* out;
};

// Reference kernels.py:1050-1076 (particle_force): penalty + damping + Coulomb.
__device__ __forceinline__ float3 pair_force(float3 n, float3 v, float c, float kn, float kd, float kf, float mu) {
    const float vn = dot3(n, v);
    const float fn = c * kn + fminf(vn, 0.0f) * kd;
    float3 vt = v - n * vn;
    const float vs = len3(vt);
    if (vs > 0.0f) vt = f3(vt.x / vs, vt.y / vs, vt.z / vs);
    const float ft = fminf(vs * kf, mu * fabsf(fn));
    return (-n) * fn - vt * ft;
}

__global__ void particle_contact_kernel(ParticleContactArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.P) return;
    float3 f = f3(0.f, 0.f, 0.f);
    if ((a.flags[i] & 1) != 0) {
        const float3 x = xyz(a.q4[i]), v = xyz(a.v4[i]);
        const float r = a.radius[i];
        const float R = r + a.max_radius + a.cohesion;
        const int x0 = cell_coord(x.x - R, a.inv_w), x1 = cell_coord(x.x + R, a.inv_w);
        const int y0 = cell_coord(x.y - R, a.inv_w), y1 = cell_coord(x.y + R, a.inv_w);
        const int z0 = cell_coord(x.z - R, a.inv_w), z1 = cell_coord(x.z + R, a.inv_w);
        // a query never spans more than dim cells per axis, so no bucket is visited twice
        const int zs = min(z1, z0 + a.dim - 1), ys = min(y1, y0 + a.dim - 1), xs = min(x1, x0 + a.dim - 1);
        for (int cz = z0; cz <= zs; ++cz)
            for (int cy = y0; cy <= ys; ++cy)
                for (int cx = x0; cx <= xs; ++cx) {
                    const int b = bucket_of(cx, cy, cz, a.dim);
                    const int lo = a.start[b], hi = a.start[b + 1];
                    for (int k = lo; k < hi; ++k) {
                        const int j = a.items[k];
                        if (j == i) continue;
                        float3 n = x - xyz(a.q4[j]);
                        const float d = len3(n);
                        if (d < 1.0e-10f) continue;
                        const float err = d - r - a.radius[j];
                        if (err <= a.cohesion) {
                            n = f3(n.x / d, n.y / d, n.z / d);
                            f = f + pair_force(n, v - xyz(a.v4[j]), err, a.ke, a.kd, a.kf, a.mu);
                        }
                    }
                }
    }
    a.out[i] = make_float4(f.x, f.y, f.z, 0.0f);
}

struct SoftContactArgs {
    int P, capacity;
    float ke, kd, kf, mu;
    const int* count;
    const int* particle;
    const float* body_pos;
    const float* body_vel;
    const float* normal;
    const float4* q4;
    const float4* v4;
    const float* radius;
    int* head;
    int* next;
    float4* force;
};

// Reference kernels.py:1198-1261: penetration = r - (x - body_pos).n; for a
// penetrating contact fn = ke pen - kd min(vn, 0) and friction capped by
// mu max(fn, 0).
__global__ void soft_contact_kernel(SoftContactArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.capacity) return;
    if (c >= *a.count) return;
    const int p = a.particle[c];
    if (p < 0 || p >= a.P) return;
    const float3 bp = f3(a.body_pos[3 * c], a.body_pos[3 * c + 1], a.body_pos[3 * c + 2]);
    const float3 bv = f3(a.body_vel[3 * c], a.body_vel[3 * c + 1], a.body_vel[3 * c + 2]);
    const float3 n = f3(a.normal[3 * c], a.normal[3 * c + 1], a.normal[3 * c + 2]);
    const float3 x = xyz(a.q4[p]), v = xyz(a.v4[p]);
    const float penetration = a.radius[p] - dot3(x - bp, n);
    if (!(penetration > 0.0f)) return;
    const float3 rel_v = v - bv;
    const float vn = dot3(rel_v, n);
    const float3 vt = rel_v - n * vn;
    const float fn = a.ke * penetration - a.kd * fminf(vn, 0.0f);
    const float vt_mag = len3(vt);
    float3 force;
    if (vt_mag > 1.0e-6f) {
        const float ft = fminf(a.kf * vt_mag, a.mu * fmaxf(0.0f, fn));
        force = n * fn - f3(vt.x / vt_mag, vt.y / vt_mag, vt.z / vt_mag) * ft;
    } else {
        force = n * fn;
    }
    a.force[c] = make_float4(force.x, force.y, force.z, 0.0f);
    a.next[c] = atomicExch(a.head + p, c);
}

}  // namespace

int particle_grid_dim(int P) {
    int d = 4;
    while (d < 128 && (int64_t)d * d * d < (int64_t)P) d *= 2;
    return d;
}

cudaError_t launch_particle_contacts(Handle& h, cudaStream_t s) {
    if (h.P == 0) return cudaSuccess;
    const float w = 2.0f * h.pmaxr + h.pcoh;
    const int nb = h.grid_dim * h.grid_dim * h.grid_dim;
    cudaError_t err = cudaMemsetAsync(h.grid_count, 0, sizeof(int) * (size_t)nb, s);
    if (err != cudaSuccess) return err;
    grid_count_kernel<<<blocks_for(h.P, 256), 256, 0, s>>>(h.P, h.q4, h.flags, 1.0f / w, h.grid_dim, h.cell_of,
                                                           h.grid_count);
    err = launch_exclusive_scan(h.grid_count, h.grid_start, nb, h.grid_part, s);
    if (err != cudaSuccess) return err;
    grid_scatter_kernel<<<blocks_for(h.P, 256), 256, 0, s>>>(h.P, h.cell_of, h.grid_start, h.grid_count,
                                                             h.grid_items);
    grid_sort_kernel<<<blocks_for(nb, 256), 256, 0, s>>>(nb, h.grid_start, h.grid_items);
    ParticleContactArgs a;
    a.P = h.P;
    a.dim = h.grid_dim;
    a.inv_w = 1.0f / w;
    a.ke = h.pke;
    a.kd = h.pkd;
    a.kf = h.pkf;
    a.mu = h.pmu;
    a.cohesion = h.pcoh;
    a.max_radius = h.pmaxr;
    a.q4 = h.q4;
    a.v4 = h.v4;
    a.radius = h.radius;
    a.flags = h.flags;
    a.start = h.grid_start;
    a.items = h.grid_items;
    a.out = h.pforce;
    particle_contact_kernel<<<blocks_for(h.P, 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_soft_contacts(Handle& h, cudaStream_t s) {
    if (h.P == 0 || h.sc_cap == 0) return cudaSuccess;
    cudaError_t err = cudaMemsetAsync(h.sc_head, 0xff, sizeof(int) * (size_t)h.P, s);
    if (err != cudaSuccess) return err;
    SoftContactArgs a;
    a.P = h.P;
    a.capacity = h.sc_cap;
    a.ke = h.ske;
    a.kd = h.skd;
    a.kf = h.skf;
    a.mu = h.smu;
    a.count = h.sc_count;
    a.particle = h.sc_particle;
    a.body_pos = h.sc_pos;
    a.body_vel = h.sc_vel;
    a.normal = h.sc_normal;
    a.q4 = h.q4;
    a.v4 = h.v4;
    a.radius = h.radius;
    a.head = h.sc_head;
    a.next = h.sc_next;
    a.force = h.sc_force;
    soft_contact_kernel<<<blocks_for(h.sc_cap, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fem
