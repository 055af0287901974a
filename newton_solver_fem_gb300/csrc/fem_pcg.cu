// Persistent block-Jacobi PCG for A dv = h f - h^2 K v with the fixed-node
// projection PAP + I - P (sm_103a, one cooperative launch per substep).
//
// Reference path (solver.py:1254-1351; implicit_predictor.py:9-41;
// fixed_particles.py:56-73, 159-168; kernels.py:1779-1868; Warp cg):
//   phase 0   rhs = f - sum_j A_ij (v_j - v_i) + spring damping, projected;
//             u = rhs - (PAP + I - P) dv           [one pass over A for both]
//   phase 1   per-scene max|rhs| -> scale (RHS normalisation); x0 = s dv,
//             r0 = s u, z0 = M r0, ||r0||^2, r0.z0, ||b||^2
//   loop      A:  p = z + beta p (recomputed on the fly at every gathered column,
//                 so no separate pass), y = (PAP + I - P) p, p.y
//             B:  x += alpha p, r -= alpha y, z = M r, ||r||^2, r.z
//   epilogue  dv = x / s; v' = v + dv; q' = q + h v'; fixed nodes restored.
// Two grid barriers per iteration.  Every cross-CTA sum is a fixed-order
// reduction of per-slice partials (no atomics on data), so results are
// deterministic and identical in every CTA.  The projection needs no column
// mask: fixed rows of r, z and p are exactly zero, so PAP p = P A p.
// Matrix layout: SELL-32 (slice of 32 consecutive rows of one scene, thread
// per row), the 9 block values split into two float4 planes and one float
// plane so that a warp streams 512 + 512 + 128 contiguous bytes per block column.
// z and p of a node share one 32-byte record, so the gather of a column
// (z_j and p_j for p = z + beta p) touches a single sector.  Iteration it reads
// record buffer it & 1; phase A hands each row's p and y to phase B through a
// staging area (shared memory when the CTA's slices fit, else a global
// buffer), and phase B writes the whole next record (z, p) at once, so every
// record write covers full sectors.
#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "fem_internal.cuh"
#include "fem_math.cuh"

namespace fem {
namespace {

struct SceneState {
    double rz;
    double atol_sq;
    double rr;
    double bb;
    float scale;
    float alpha;
    float beta;
    int active;
    int iters;
    int zero;
    int primed;  // single-reduction variant: the first SpMV (w0 = A u0) has been reduced
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed_int(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier over a monotone counter (zeroed before the launch), entered by
// one thread per CTA after a CTA or warp barrier has ordered the CTA's writes
// before it.  The arrival is a release reduction, so those writes are visible
// at GPU scope before it; the wait is an acquire load, so the other CTAs'
// writes are visible after it.  The wait is bounded: it gives up after
// limit_ns nanoseconds, or as soon as another CTA has given up, and returns 0.
__device__ __forceinline__ int arrive_and_wait(unsigned* counter, unsigned nblocks, unsigned& epoch, int* status,
                                               long long limit_ns) {
    epoch += 1;
    const unsigned target = epoch * nblocks;
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(counter) : "memory");
    const unsigned long long t0 = global_ns();
    unsigned spins = 0;
    while ((int)(ld_acquire(counter) - target) < 0) {  // wrap-safe: the counter only grows
        if ((++spins & 63u) == 1u) {  // first spin, then every 64th
            if ((ld_relaxed_int(status) & kStatusTimeout) != 0 || (long long)(global_ns() - t0) >= limit_ns) {
                atomicOr(status, kStatusTimeout);
                return 0;
            }
        }
    }
    return 1;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}
__device__ __forceinline__ float3 bmul(float4 a, float4 b, float c, float3 p) {
    return f3(a.x * p.x + a.y * p.y + a.z * p.z, a.w * p.x + b.x * p.y + b.y * p.z, b.z * p.x + b.w * p.y + c * p.z);
}

__device__ __forceinline__ float3 minv_mul(const float* __restrict__ m, int row, float3 r) {
    const float* b = m + 9 * (size_t)row;
    return f3(b[0] * r.x + b[1] * r.y + b[2] * r.z, b[3] * r.x + b[4] * r.y + b[5] * r.z,
              b[6] * r.x + b[7] * r.y + b[8] * r.z);
}

__device__ __forceinline__ float3 load3(const float* p, int i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void store3(float* p, int i, float3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

// Same expression at the owner and at every gathering neighbour, so the
// recomputed search direction is bit-identical everywhere.
__device__ __forceinline__ float3 next_p(float4 z, float4 p, float beta) {
    return f3(fmaf(beta, p.x, z.x), fmaf(beta, p.y, z.y), fmaf(beta, p.z, z.z));
}

// ---------------------------------------------------------------------------
// Matrix stream loads.  The matrix is read-only during the kernel, so it goes
// through the non-coherent path without L1 allocation, with an L2 eviction
// policy per slice: the first `resident_slices` slices are loaded evict_last
// so that they stay in L2 from one CG iteration to the next, the rest
// evict_first so that streaming them does not displace the resident part or
// the CG vectors.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long policy_evict_last() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ unsigned long long policy_evict_first() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
// Bulk L2 prefetch (no register or shared-memory destination): the address and
// the size are multiples of 16 bytes.
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

__device__ __forceinline__ float4 ld_mat4(const float4* p, unsigned long long pol) {
    float4 v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float ld_mat1(const float* p, unsigned long long pol) {
    float v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ int ld_col(const int* p, unsigned long long pol) {
    int v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ int ld_dcol(const short* p, unsigned long long pol) {
    unsigned short v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
    return (int)(short)v;
}

struct Entry {
    float4 A, B;
    float C;
    int j;
};

// The 16-bit column offset of entry e, loaded only when `load` (warp-uniform);
// otherwise `shared`, the offset every row of the slice has at this k.
__device__ __forceinline__ int ld_dcol_unless(const short* p, unsigned long long pol, bool load, short shared) {
    unsigned short v = (unsigned short)shared;
    asm volatile(
        "{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t"
        "@q ld.global.nc.L1::no_allocate.L2::cache_hint.b16 %0, [%1], %3;\n\t}"
        : "+h"(v)
        : "l"(p), "r"((unsigned)load), "l"(pol));
    return (int)(short)v;
}

// Column storage of the SpMV (the kernel's CM template parameter): 0 the 32-bit
// column; 1 the row plus a 16-bit offset, which saves 2 of the 40 bytes a block
// costs; 2 the same, except that at the slots k < 64 where every row of the
// slice has the same offset (bit k of the slice's mask) it is read once from
// shared memory instead of per row.
struct SliceCols {
    unsigned long long mask;  // CM 2: uniform slots
    const short* val;         // CM 2: [64] their offsets (shared memory)
};

// One stored block and its column.
template <int CM>
__device__ __forceinline__ Entry load_entry(const PcgArgs& a, size_t e, int k, int row, const SliceCols& sc,
                                            unsigned long long pol) {
    Entry m;
    m.A = ld_mat4(a.valA + e, pol);
    m.B = ld_mat4(a.valB + e, pol);
    m.C = ld_mat1(a.valC + e, pol);
    if (CM == 2) {
        const bool uni = k < 64 && ((sc.mask >> k) & 1ull);
        m.j = row + ld_dcol_unless(a.dcol + e, pol, !uni, uni ? sc.val[k] : (short)0);
    } else {
        m.j = CM == 1 ? row + ld_dcol(a.dcol + e, pol) : ld_col(a.scol + e, pol);
    }
    return m;
}

// p_j = z_j (first iteration) or z_j + beta p_j from record buffer rec.
template <bool FIRST>
__device__ __forceinline__ float3 gather_p(const float4* rec, int j, float beta) {
    const float4* q = rec + 2 * (size_t)j;
    if (FIRST) return xyz(q[0]);
    return next_p(q[0], q[1], beta);
}

// y_row = sum_k A_k p_{j_k}, with p = z (first iteration) or z + beta p_old.
// U block columns are loaded before any is used, so U entries (and then U
// gathers) are in flight per thread; the sum keeps the k order of U = 1.
template <int U, int CM, bool FIRST>
__device__ __forceinline__ float3 row_times_p(const PcgArgs& a, int base, int len, int lane, int row,
                                              const SliceCols& sc, const float4* rec, float beta,
                                              unsigned long long pol) {
    float3 acc = f3(0.f, 0.f, 0.f);
    int k = 0;
    if (U > 1) {
        for (; k + U <= len; k += U) {
            Entry m[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                m[u] = load_entry<CM>(a, (size_t)(base + k + u) * kSlice + lane, k + u, row, sc, pol);
            float3 p[U];
#pragma unroll
            for (int u = 0; u < U; ++u) p[u] = gather_p<FIRST>(rec, m[u].j, beta);
#pragma unroll
            for (int u = 0; u < U; ++u) acc = acc + bmul(m[u].A, m[u].B, m[u].C, p[u]);
        }
    }
    for (; k < len; ++k) {
        Entry m = load_entry<CM>(a, (size_t)(base + k) * kSlice + lane, k, row, sc, pol);
        float3 p = gather_p<FIRST>(rec, m.j, beta);
        acc = acc + bmul(m.A, m.B, m.C, p);
    }
    return acc;
}

// Single-reduction (Chronopoulos-Gear) records: node j's (u_j, Mw_j, Ms_j) as 3 float4 = (u.xyz, mw.x),
// (mw.yz, ms.xy), (ms.z, -, -, -).  The next preconditioned residual u' = M r' = u - alpha (Mw + beta Ms)
// follows from the record alone, so a gathering row recomputes it with the same expression the owner
// uses (bit-identical everywhere) instead of waiting at a second grid barrier for the owner to write it.
__device__ __forceinline__ float3 next_u(float4 r0, float4 r1, float r2x, float alpha, float beta, float3& t) {
    t = f3(fmaf(beta, r1.z, r0.w), fmaf(beta, r1.w, r1.x), fmaf(beta, r2x, r1.y));  // M s = Mw + beta Ms
    return f3(fmaf(-alpha, t.x, r0.x), fmaf(-alpha, t.y, r0.y), fmaf(-alpha, t.z, r0.z));
}
template <bool PRIME>
__device__ __forceinline__ float3 gather_u(const float4* rec, int j, float alpha, float beta) {
    const float4* q = rec + 3 * (size_t)j;
    const float4 r0 = q[0];
    if (PRIME) return xyz(r0);
    const float4 r1 = q[1];
    const float r2x = reinterpret_cast<const float*>(q + 2)[0];
    float3 t;
    return next_u(r0, r1, r2x, alpha, beta, t);
}

// w_row = sum_k A_k u'_{j_k} (the single-reduction variant's SpMV), U block columns in flight.
template <int U, int CM, bool PRIME>
__device__ __forceinline__ float3 row_times_u(const PcgArgs& a, int base, int len, int lane, int row,
                                              const SliceCols& sc, const float4* rec, float alpha, float beta,
                                              unsigned long long pol) {
    float3 acc = f3(0.f, 0.f, 0.f);
    int k = 0;
    if (U > 1) {
        for (; k + U <= len; k += U) {
            Entry m[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                m[u] = load_entry<CM>(a, (size_t)(base + k + u) * kSlice + lane, k + u, row, sc, pol);
            float3 g[U];
#pragma unroll
            for (int u = 0; u < U; ++u) g[u] = gather_u<PRIME>(rec, m[u].j, alpha, beta);
#pragma unroll
            for (int u = 0; u < U; ++u) acc = acc + bmul(m[u].A, m[u].B, m[u].C, g[u]);
        }
    }
    for (; k < len; ++k) {
        Entry m = load_entry<CM>(a, (size_t)(base + k) * kSlice + lane, k, row, sc, pol);
        float3 g = gather_u<PRIME>(rec, m.j, alpha, beta);
        acc = acc + bmul(m.A, m.B, m.C, g);
    }
    return acc;
}

// Prologue pass: cv = sum_k A_k (v_j - v_i) and ax = sum_k A_k x_j in one read of the row.
template <int U, int CM>
__device__ __forceinline__ void row_predictor(const PcgArgs& a, int base, int len, int lane, int row,
                                              const SliceCols& sc, float3 vi, float3& cv, float3& ax,
                                              unsigned long long pol) {
    int k = 0;
    if (U > 1) {
        for (; k + U <= len; k += U) {
            Entry m[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                m[u] = load_entry<CM>(a, (size_t)(base + k + u) * kSlice + lane, k + u, row, sc, pol);
            float3 vj[U], xj[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                vj[u] = xyz(a.v4[m[u].j]);
                xj[u] = xyz(a.x[m[u].j]);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                cv = cv + bmul(m[u].A, m[u].B, m[u].C, vj[u] - vi);
                ax = ax + bmul(m[u].A, m[u].B, m[u].C, xj[u]);
            }
        }
    }
    for (; k < len; ++k) {
        Entry m = load_entry<CM>(a, (size_t)(base + k) * kSlice + lane, k, row, sc, pol);
        float3 vj = xyz(a.v4[m.j]), xj = xyz(a.x[m.j]);
        cv = cv + bmul(m.A, m.B, m.C, vj - vi);
        ax = ax + bmul(m.A, m.B, m.C, xj);
    }
}

struct Smem {
    float* part;      // [L * 3] slice partials
    SceneState* st;   // [S]
    float* tot;       // [S * 3] per-scene totals of the last reduction
    float4* stage;    // [L * 32 * 2] (p, y) per row, when staged in shared memory
    int* segb;        // [L + 1] bounds (positions in the CTA's slice list) of its per-scene segments,
                      // then [L] where each segment's partials go in the segment buffer
    int* sseg;        // [S + 1] first segment of every scene (copy of scene_seg0)
    float* res;       // [L * 32 * res_floats] resident row state (x, r, z[, inverse diagonal block])
    int4* slc;        // [L] this CTA's slices: (first row, row count, scene | kResidentSlice, SELL base)
    unsigned long long* kmask;  // [L] column mode 2: uniform-offset slots of each slice
    short* kval;                // [L * 64] column mode 2: their offsets
    unsigned* rinfo;  // [L * 32] row length | fixed bit of this CTA's rows
    int nsc;          // scenes (segments) this CTA covers
};

// Resident row state, per row of the CTA: x (0-2), r (3-5), z (6-8) and, in
// layout 2, the block-Jacobi inverse (9-17; layout 1 reads it from global
// memory).  With it, the x/r/z update reads and writes shared memory only; the
// (z, p) record is still written for the gathers.
// Single-reduction variant (V = 1): x (0-2), r (3-5), p (6-8), s (9-11), w (12-14) and, in layout 2,
// the inverse (15-23).
__host__ __device__ __forceinline__ int res_floats(int layout, int V = 0) {
    return V == 1 ? (layout == 2 ? 24 : 15) : (layout == 2 ? 18 : 9);
}
__host__ __device__ __forceinline__ int res_minv_offset(int V) { return V == 1 ? 15 : 9; }

// The resident state of row `row` (lane `lane` of slice `sl`).
__device__ __forceinline__ float* res_slot(const Smem& sm, int sl, int first, int lane, int layout, int V = 0) {
    return sm.res + (size_t)((sl - first) * kSlice + lane) * res_floats(layout, V);
}
__device__ __forceinline__ float3 res3(const float* s, int k) { return f3(s[k], s[k + 1], s[k + 2]); }
__device__ __forceinline__ void res3_store(float* s, int k, float3 v) {
    s[k] = v.x;
    s[k + 1] = v.y;
    s[k + 2] = v.z;
}
__device__ __forceinline__ float3 res_minv_mul(const float* s, float3 r, int off = 9) {
    const float* b = s + off;
    return f3(b[0] * r.x + b[1] * r.y + b[2] * r.z, b[3] * r.x + b[4] * r.y + b[5] * r.z,
              b[6] * r.x + b[7] * r.y + b[8] * r.z);
}

// Scenes up to this count are reduced lane-parallel over their segments by one
// warp; more scenes are reduced one scene per thread by the whole CTA.
constexpr int kWarpReducedScenes = 4;

// The (p, y) staging of a CTA goes to shared memory when it needs at most
// this many bytes per warp of the CTA (1 KB per slice).
constexpr int kStageBytesPerWarp = 6 * 1024;
__host__ __device__ __forceinline__ bool stage_in_smem(int L, int threads) {
    return (size_t)L * kSlice * 2 * sizeof(float4) <= (size_t)kStageBytesPerWarp * (threads / 32);
}

// Byte offsets of the dynamic shared memory sections; every section starts on
// a 16-byte boundary (the staging area holds float4).  One definition serves
// the kernel and the host-side size.
struct SmemLayout {
    size_t part, st, tot, segb, sseg, slc, kmask, kval, rinfo, stage, res, total;
};
__host__ __device__ __forceinline__ size_t align16(size_t n) { return (n + 15) & ~(size_t)15; }
__host__ __device__ __forceinline__ SmemLayout smem_layout(int L, int S, bool stage, int resident, bool uni,
                                                             int V = 0) {
    SmemLayout m;
    m.part = 0;
    m.st = m.part + align16((size_t)L * 3 * sizeof(float));
    m.tot = m.st + align16((size_t)S * sizeof(SceneState));
    m.segb = m.tot + align16((size_t)S * 3 * sizeof(float));
    m.sseg = m.segb + align16((size_t)(2 * L + 1) * sizeof(int));
    m.slc = m.sseg + align16((size_t)(S + 1) * sizeof(int));
    m.kmask = m.slc + align16((size_t)L * sizeof(int4));
    m.kval = m.kmask + (uni ? align16((size_t)L * sizeof(unsigned long long)) : 0);
    m.rinfo = m.kval + (uni ? align16((size_t)L * 64 * sizeof(short)) : 0);
    m.stage = m.rinfo + align16((size_t)L * kSlice * sizeof(unsigned));
    m.res = m.stage + (stage ? (size_t)L * kSlice * 2 * sizeof(float4) : 0);
    m.total = m.res + (resident ? (size_t)L * kSlice * res_floats(resident, V) * sizeof(float) : 0);
    return m;
}

// Where row `row` (lane `lane` of slice `sl`) stages its p and y between the phases.
__device__ __forceinline__ float4* stage_slot(const PcgArgs& a, const Smem& sm, int sl, int first, int lane, int row) {
    return a.stage_smem ? sm.stage + 2 * ((sl - first) * kSlice + lane) : a.stage + 2 * (size_t)row;
}

// One grid-wide reduction step, entered by every thread of the CTA once the
// slice partials of the current phase are in sm.part:
//   1. warp 0 writes this CTA's per-scene segment partials (sum or max of its
//      slices of the scene: lane-strided, then a fixed xor butterfly) to buf;
//   2. one thread arrives at the grid barrier and waits for every CTA;
//   3. the per-scene totals over all segments (each lane sums its strided
//      segments in ascending order, then the butterfly) go to sm.tot, and
//      upd(s) runs once per scene: on lane s of warp 0 for a few scenes, else
//      on the thread that formed scene s's totals.
// Every CTA forms bit-identical totals.  Consecutive reductions alternate
// between two buffers: a CTA that races ahead can only write a buffer again
// after the next barrier, which every CTA reaches only once it has finished
// reading that buffer's previous contents.  Partials and totals are float,
// like the reference solver's float32 dot products; the order is fixed, so
// results are deterministic.  When s_any is given it is cleared on entry (for
// the updates to set).  Returns false after a timed-out wait.
constexpr int kSegLoadBatch = 8;  // segment partials a lane loads before adding them
constexpr int kSegmentsPerWarp0 = 2;  // segments warp 0 writes alone
constexpr int kResidentSlice = 1 << 30;  // slice table scene field: the slice's blocks are loaded evict_last

// Segment t's partials (sum or max over its slices: lane-strided, then a fixed
// xor butterfly) to its slot of the segment buffer; entered by a whole warp.
__device__ __forceinline__ void write_segment(const PcgArgs& a, const Smem& sm, float* buf, int nv, bool is_max,
                                              int first, int t, int lane) {
    const int lo = sm.segb[t], hi = sm.segb[t + 1];
    for (int k = 0; k < nv; ++k) {
        float acc = 0.f;
        for (int sl = lo + lane; sl < hi; sl += 32) {
            const float v = sm.part[(sl - first) * 3 + k];
            acc = is_max ? fmaxf(acc, v) : acc + v;
        }
        acc = is_max ? warp_max(acc) : warp_sum(acc);
        if (lane == 0) buf[(size_t)sm.segb[a.slices_per_cta + 1 + t] * 3 + k] = acc;
    }
}

template <class Update>
__device__ bool reduce_across_grid(const PcgArgs& a, const Smem& sm, float* buf, int nv, bool is_max, int first,
                                   int last, unsigned& epoch, int* s_ok, int* s_any, Update upd) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int S = a.nscenes;
    if (threadIdx.x == 0 && s_any != nullptr) *s_any = 0;
    __syncthreads();  // slice partials complete, activity flag cleared
    // many segments: all warps write them, and a CTA barrier orders the writes
    // before the arrival
    const bool spread = sm.nsc > kSegmentsPerWarp0;
    if (spread) {
        for (int t = warp; t < sm.nsc; t += (int)(blockDim.x >> 5)) write_segment(a, sm, buf, nv, is_max, first, t, lane);
        __syncthreads();
    }
    if (warp == 0) {
        if (!spread)
            for (int t = 0; t < sm.nsc; ++t) write_segment(a, sm, buf, nv, is_max, first, t, lane);
        __syncwarp();
        int ok = 1;
        // a one-CTA grid needs no grid barrier: the CTA barrier or warp order above already orders
        // every partial before it is read
        if (lane == 0 && gridDim.x > 1) ok = arrive_and_wait(a.barrier, gridDim.x, epoch, a.status, a.limit_ns);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (ok && S <= kWarpReducedScenes) {
            for (int sc = 0; sc < S; ++sc) {
                const int lo = sm.sseg[sc], hi = sm.sseg[sc + 1];
                float acc[3] = {0.f, 0.f, 0.f};
                for (int g0 = lo + lane; g0 < hi; g0 += 32 * kSegLoadBatch) {
                    float v[kSegLoadBatch][3];
#pragma unroll
                    for (int u = 0; u < kSegLoadBatch; ++u) {
                        const int g = g0 + 32 * u;
                        for (int k = 0; k < nv; ++k) v[u][k] = g < hi ? __ldcg(buf + (size_t)g * 3 + k) : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < kSegLoadBatch; ++u)
                        if (g0 + 32 * u < hi)
                            for (int k = 0; k < nv; ++k) acc[k] = is_max ? fmaxf(acc[k], v[u][k]) : acc[k] + v[u][k];
                }
                for (int k = 0; k < nv; ++k) {
                    const float t = is_max ? warp_max(acc[k]) : warp_sum(acc[k]);
                    if (lane == 0) sm.tot[sc * 3 + k] = t;
                }
            }
            __syncwarp();
            if (lane < S) upd(lane);
        }
        if (lane == 0) *s_ok = ok;
    }
    if (S > kWarpReducedScenes) {
        __syncthreads();
        if (!*s_ok) return false;
        for (int sc = threadIdx.x; sc < S; sc += blockDim.x) {
            const int lo = sm.sseg[sc], hi = sm.sseg[sc + 1];
            for (int k = 0; k < nv; ++k) {
                float acc = 0.f;
                for (int g = lo; g < hi; ++g) {
                    const float v = __ldcg(buf + (size_t)g * 3 + k);
                    acc = is_max ? fmaxf(acc, v) : acc + v;
                }
                sm.tot[sc * 3 + k] = acc;
            }
            upd(sc);
        }
    }
    __syncthreads();
    return *s_ok != 0;
}

// A CTA's warps take its slices round-robin.  When the last round keeps at most
// tail_prefetch percent of the warps busy (and its second round is also its
// last), those few warps cannot keep enough loads in flight to cover DRAM
// latency; so the last warp, idle in that round, requests the
// round's slices (one contiguous range per value/column plane) into L2 while
// the first round streams.  The bytes are the same; the last round then reads
// from L2.  SELL planes start every slice on a 32-entry boundary, so every range
// is 16-byte aligned; requests are 32 KB.
constexpr unsigned kPrefetchChunk = 32 * 1024;
__device__ __forceinline__ void prefetch_range(const void* base, size_t bytes, int lane) {
    const char* p = static_cast<const char*>(base);
    for (size_t off = (size_t)lane * kPrefetchChunk; off < bytes; off += 32 * (size_t)kPrefetchChunk)
        prefetch_l2(p + off, (unsigned)min((size_t)kPrefetchChunk, bytes - off));
}
__device__ __noinline__ void prefetch_last_round(const PcgArgs& a, const Smem& sm, int first, int last, int W,
                                                 int lane) {
    const int n = last - first;
    if (n <= W || 100 * (n - W) > a.tail_prefetch * W) return;
    const int e0 = sm.slc[W].w * kSlice, e1 = __ldg(a.slice_ptr + last) * kSlice;
    const size_t m = (size_t)(e1 - e0);
    prefetch_range(a.valA + e0, m * sizeof(float4), lane);
    prefetch_range(a.valB + e0, m * sizeof(float4), lane);
    prefetch_range(a.valC + e0, m * sizeof(float), lane);
    if (a.dcol != nullptr) prefetch_range(a.dcol + e0, m * sizeof(short), lane);
    else prefetch_range(a.scol + e0, m * sizeof(int), lane);
}

__device__ __forceinline__ float rhs_scale(float maximum) {
    // kernels.py:1785-1793
    float scale = 1.0f;
    if (maximum > 0.0f && maximum < 1.0e-12f) scale = fminf(1.0f / maximum, 1.0e30f);
    return scale;
}

template <int U, int CM, int V>
__global__ void __launch_bounds__(kPcgMaxThreads, 1) pcg_kernel(PcgArgs a) {
    const unsigned long long pol_last = policy_evict_last();
    const unsigned long long pol_first = policy_evict_first();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_ok;
    __shared__ int s_any;
    const int S = a.nscenes;
    const int L = a.slices_per_cta;
    Smem sm;
    const SmemLayout lay = smem_layout(L, S, a.stage_smem != 0, a.resident, CM == 2, V);
    sm.part = reinterpret_cast<float*>(smem_raw + lay.part);
    sm.st = reinterpret_cast<SceneState*>(smem_raw + lay.st);
    sm.tot = reinterpret_cast<float*>(smem_raw + lay.tot);
    sm.stage = reinterpret_cast<float4*>(smem_raw + lay.stage);
    sm.segb = reinterpret_cast<int*>(smem_raw + lay.segb);
    sm.sseg = reinterpret_cast<int*>(smem_raw + lay.sseg);
    sm.res = reinterpret_cast<float*>(smem_raw + lay.res);
    sm.slc = reinterpret_cast<int4*>(smem_raw + lay.slc);
    sm.rinfo = reinterpret_cast<unsigned*>(smem_raw + lay.rinfo);
    sm.kmask = reinterpret_cast<unsigned long long*>(smem_raw + lay.kmask);
    sm.kval = reinterpret_cast<short*>(smem_raw + lay.kval);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int first = a.cta_slice0[blockIdx.x];
    const int last = a.cta_slice0[blockIdx.x + 1];
    __shared__ unsigned long long s_t0;  // SpMV-phase start (speed calibration only)
    // Launch-constant reduction tables, staged once (the first grid reduction's
    // CTA barrier orders these writes before their use).
    {
        const int segbase = a.cta_seg_base[blockIdx.x];
        sm.nsc = a.cta_seg_base[blockIdx.x + 1] - segbase;
        for (int t = threadIdx.x; t <= sm.nsc; t += blockDim.x) {
            sm.segb[t] = t == sm.nsc ? last : a.seg_start[segbase + t];
            if (t < sm.nsc) sm.segb[L + 1 + t] = a.seg_pos[segbase + t];
        }
        for (int t = threadIdx.x; t <= S; t += blockDim.x) sm.sseg[t] = a.scene_seg0[t];
        for (int t = threadIdx.x; t < last - first; t += blockDim.x) {
            const int g = a.cta_list[first + t];
            const int2 m = a.slice_meta[g];
            sm.slc[t] = make_int4(m.x, m.y, a.slice_scene[g] | (g < a.resident_slices ? kResidentSlice : 0),
                                  a.slice_ptr[g]);
            if (CM == 2) sm.kmask[t] = a.slice_kmask[g];
        }
        if (CM == 2)
            for (int t = threadIdx.x; t < (last - first) * 64; t += blockDim.x)
                sm.kval[t] = a.slice_kval[(size_t)a.cta_list[first + t / 64] * 64 + t % 64];
    }
    __syncthreads();  // the slice table is complete before the row table reads it
    for (int t = threadIdx.x; t < (last - first) * kSlice; t += blockDim.x) {
        const int4 m = sm.slc[t / kSlice];
        const int lane_t = t % kSlice;
        sm.rinfo[t] = lane_t < m.y ? a.row_info[m.x + lane_t] : 0u;
    }
    __syncthreads();
    unsigned epoch = 0;
    const float h = a.dt;
    auto slice_cols = [&](int sl) {
        return CM == 2 ? SliceCols{sm.kmask[sl - first], sm.kval + 64 * (sl - first)} : SliceCols{0ull, nullptr};
    };

    // ---------------- phase 0: RHS (predictor, springs, projection) and u = rhs - A x0
    if (a.tail_prefetch && a.contiguous && warp == W - 1) prefetch_last_round(a, sm, first, last, W, lane);
    for (int sl = first + warp; sl < last; sl += W) {
        const int4 sl4 = sm.slc[sl - first];
        const int2 meta = make_int2(sl4.x, sl4.y);
        float mx = 0.0f;
        if (lane < meta.y) {
            int row = meta.x + lane;
            unsigned info = sm.rinfo[(sl - first) * kSlice + lane];
            float3 rhs = f3(0.f, 0.f, 0.f), u = f3(0.f, 0.f, 0.f);
            if (a.solve_rhs != nullptr) {
                // solve mode: A x = b, b given (projected at fixed rows), from x0 = 0 or the packed x
                if (!(info & kFixedBit)) rhs = load3(a.solve_rhs, row);
                u = rhs;
                if (a.solve_warm && !(info & kFixedBit)) {
                    float3 cv = f3(0.f, 0.f, 0.f), ax = f3(0.f, 0.f, 0.f);
                    row_predictor<U, CM>(a, sl4.w, (int)(info & ~kFixedBit), lane, row, slice_cols(sl), xyz(a.v4[row]),
                                         cv, ax, (sl4.z & kResidentSlice) ? pol_last : pol_first);
                    u = rhs - ax;
                }
            } else {
                if (!(info & kFixedBit)) {
                    int len = (int)(info & ~kFixedBit);
                    float3 vi = xyz(a.v4[row]);
                    float3 cv = f3(0.f, 0.f, 0.f), ax = f3(0.f, 0.f, 0.f);
                    row_predictor<U, CM>(a, sl4.w, len, lane, row, slice_cols(sl), vi, cv, ax,
                                         (sl4.z & kResidentSlice) ? pol_last : pol_first);
                    rhs = load3(a.f_ws, row) - cv;
                    for (int e = a.spring_ptr[row]; e < a.spring_ptr[row + 1]; ++e) {
                        int ent = a.spring_ent[e];
                        int s = ent >> 1;
                        int ia = a.spring_idx[2 * s], ib = a.spring_idx[2 * s + 1];
                        if (ia < 0 || ib < 0) continue;
                        float3 corr = (xyz(a.v4[ia]) - xyz(a.v4[ib])) * (h * a.spring_kd[s]);
                        rhs = (ent & 1) ? rhs - corr : rhs + corr;
                    }
                    u = rhs - ax;
                }
                store3(a.f_ws, row, rhs);
            }
            if (a.resident) res3_store(res_slot(sm, sl, first, lane, a.resident, V), 3, u);
            else a.r[row] = f4(u);
            mx = fmaxf(fabsf(rhs.x), fmaxf(fabsf(rhs.y), fabsf(rhs.z)));
        }
        mx = warp_max(mx);
        if (lane == 0) sm.part[(sl - first) * 3] = mx;
    }
    float* const buf0 = a.seg_part;
    float* const buf1 = a.seg_part + (size_t)a.nseg * 3;
    auto set_scale = [&](int s) {
        const float mxs = sm.tot[s * 3];
        sm.st[s].scale = rhs_scale(mxs);
        sm.st[s].zero = mxs == 0.0f;
    };
    if (!reduce_across_grid(a, sm, buf0, 1, true, first, last, epoch, &s_ok, nullptr, set_scale)) return;

    // ---------------- phase 1: normalise, initial residual and preconditioned residual
    for (int sl = first + warp; sl < last; sl += W) {
        const int4 sl4 = sm.slc[sl - first];
        const int2 meta = make_int2(sl4.x, sl4.y);
        const SceneState& st = sm.st[sl4.z & ~kResidentSlice];
        float rr = 0.f, rz = 0.f, bb = 0.f;
        if (lane < meta.y) {
            int row = meta.x + lane;
            float sc = st.scale;
            float3 x = f3(0.f, 0.f, 0.f), r = f3(0.f, 0.f, 0.f);
            float* rs = a.resident ? res_slot(sm, sl, first, lane, a.resident, V) : nullptr;
            if (!st.zero) {
                if (a.solve_rhs == nullptr || a.solve_warm) x = xyz(a.x[row]) * sc;  // else solve mode starts from zero
                r = (a.resident ? res3(rs, 3) : xyz(a.r[row])) * sc;
            }
            float3 b;
            if (a.solve_rhs != nullptr)
                b = (sm.rinfo[(sl - first) * kSlice + lane] & kFixedBit) ? f3(0.f, 0.f, 0.f)
                                                                         : load3(a.solve_rhs, row) * sc;
            else
                b = load3(a.f_ws, row) * sc;
            float3 z;
            const int mo = res_minv_offset(V);
            if (a.resident) {
                if (a.resident == 2) {
                    for (int k = 0; k < 9; ++k) rs[mo + k] = a.minv[9 * (size_t)row + k];
                    z = res_minv_mul(rs, r, mo);
                } else {
                    z = minv_mul(a.minv, row, r);
                }
                res3_store(rs, 0, x);
                res3_store(rs, 3, r);
                if (V == 0) {
                    res3_store(rs, 6, z);
                } else {  // p, s, w start at zero
                    res3_store(rs, 6, f3(0.f, 0.f, 0.f));
                    res3_store(rs, 9, f3(0.f, 0.f, 0.f));
                    res3_store(rs, 12, f3(0.f, 0.f, 0.f));
                }
            } else {
                z = minv_mul(a.minv, row, r);
                a.x[row] = f4(x);
                a.r[row] = f4(r);
                if (V == 1) {
                    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
                    a.p4[row] = zero4;
                    a.s4[row] = zero4;
                    a.w4[row] = zero4;
                }
            }
            if (V == 0) {
                a.zp0[2 * (size_t)row] = f4(z);
                a.zp0[2 * (size_t)row + 1] = f4(f3(0.f, 0.f, 0.f));  // full record; p unused in the first iteration
            } else {  // record (u0, Mw = 0, Ms = 0) for the first SpMV, w0 = A u0
                a.rec0[3 * (size_t)row] = make_float4(z.x, z.y, z.z, 0.f);
                a.rec0[3 * (size_t)row + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
                a.rec0[3 * (size_t)row + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            rr = dot3(r, r);
            rz = dot3(r, z);
            bb = dot3(b, b);
        }
        rr = warp_sum(rr);
        rz = warp_sum(rz);
        bb = warp_sum(bb);
        if (lane == 0) {
            float* p = sm.part + (sl - first) * 3;
            p[0] = rr; p[1] = rz; p[2] = bb;
        }
    }
    auto start_cg = [&](int s) {
        SceneState& st = sm.st[s];
        st.rr = sm.tot[s * 3];
        st.rz = sm.tot[s * 3 + 1];
        st.bb = sm.tot[s * 3 + 2];
        st.atol_sq = (double)a.tol * (double)a.tol * st.bb;
        st.iters = 0;
        st.beta = 0.0f;
        st.alpha = 0.0f;
        st.primed = 0;
        st.active = (st.rr > st.atol_sq) && (a.maxiter > 0);
        if (!isfinite(st.rr)) {
            st.active = 0;
            atomicOr(a.status, kStatusNonFinite);
        }
        if (st.active) atomicOr(&s_any, 1);
    };
    if (!reduce_across_grid(a, sm, buf1, 3, false, first, last, epoch, &s_ok, &s_any, start_cg)) return;

    // ---------------- CG iterations
    if constexpr (V == 0) {
    for (int it = 0; s_any; ++it) {
        const float4* rec = (it & 1) ? a.zp1 : a.zp0;  // z and p of this iteration
        float4* rec_next = (it & 1) ? a.zp0 : a.zp1;   // (z, p) for the next, written by phase B
        // phase A: p = z + beta p, y = (PAP + I - P) p, partial p.y
        if (a.cta_time != nullptr && threadIdx.x == 0) s_t0 = global_ns();
        if (a.tail_prefetch && a.contiguous && warp == W - 1) prefetch_last_round(a, sm, first, last, W, lane);
        for (int sl = first + warp; sl < last; sl += W) {
            const int4 sl4 = sm.slc[sl - first];
            const int2 meta = make_int2(sl4.x, sl4.y);
            const SceneState& st = sm.st[sl4.z & ~kResidentSlice];
            float pap = 0.f;
            if (st.active && lane < meta.y) {
                int row = meta.x + lane;
                unsigned info = sm.rinfo[(sl - first) * kSlice + lane];
                const bool firstit = st.iters == 0;
                const float beta = st.beta;
                float3 pc;
                if (a.resident) {  // own z resident, previous p in this row's staging slot
                    const float3 zi = res3(res_slot(sm, sl, first, lane, a.resident), 6);
                    pc = firstit ? zi : next_p(f4(zi), stage_slot(a, sm, sl, first, lane, row)[0], beta);
                } else {
                    const float4 zi = rec[2 * (size_t)row];
                    pc = firstit ? xyz(zi) : next_p(zi, rec[2 * (size_t)row + 1], beta);
                }
                float3 acc = pc;  // fixed rows: identity (their p is zero)
                if (!(info & kFixedBit)) {
                    int len = (int)(info & ~kFixedBit);
                    int base = sl4.w;
                    unsigned long long pol = (sl4.z & kResidentSlice) ? pol_last : pol_first;
                    const SliceCols sc = slice_cols(sl);
                    acc = firstit ? row_times_p<U, CM, true>(a, base, len, lane, row, sc, rec, beta, pol)
                                  : row_times_p<U, CM, false>(a, base, len, lane, row, sc, rec, beta, pol);
                }
                float4* stg = stage_slot(a, sm, sl, first, lane, row);
                stg[0] = f4(pc);
                stg[1] = f4(acc);
                pap = dot3(pc, acc);
            }
            pap = warp_sum(pap);
            if (lane == 0) sm.part[(sl - first) * 3] = pap;
        }
        auto set_alpha = [&](int s) {
            SceneState& st = sm.st[s];
            if (st.active) st.alpha = (float)(st.rz / sm.tot[s * 3]);
        };
        if (a.cta_time != nullptr) {  // speed calibration: this CTA's SpMV-phase time
            __syncthreads();
            if (threadIdx.x == 0) {
                a.cta_time[2 * blockIdx.x] += global_ns() - s_t0;
                a.cta_time[2 * blockIdx.x + 1] += 1;
            }
        }
        if (!reduce_across_grid(a, sm, buf0, 1, false, first, last, epoch, &s_ok, nullptr, set_alpha)) return;
        // phase B: x += alpha p, r -= alpha y, z = M r, partial r.r and r.z
        for (int sl = first + warp; sl < last; sl += W) {
            const int4 sl4 = sm.slc[sl - first];
            const int2 meta = make_int2(sl4.x, sl4.y);
            const SceneState& st = sm.st[sl4.z & ~kResidentSlice];
            float rr = 0.f, rz = 0.f;
            if (st.active && lane < meta.y) {
                int row = meta.x + lane;
                float alpha = st.alpha;
                const float4* stg = stage_slot(a, sm, sl, first, lane, row);
                float3 p = xyz(stg[0]), yv = xyz(stg[1]);
                float* rs = a.resident ? res_slot(sm, sl, first, lane, a.resident) : nullptr;
                float3 x = a.resident ? res3(rs, 0) : xyz(a.x[row]);
                float3 r = a.resident ? res3(rs, 3) : xyz(a.r[row]);
                x = x + p * alpha;
                r = r - yv * alpha;
                float3 z;
                if (a.resident) {
                    z = a.resident == 2 ? res_minv_mul(rs, r) : minv_mul(a.minv, row, r);
                    res3_store(rs, 0, x);
                    res3_store(rs, 3, r);
                    res3_store(rs, 6, z);
                } else {
                    z = minv_mul(a.minv, row, r);
                    a.x[row] = f4(x);
                    a.r[row] = f4(r);
                }
                rec_next[2 * (size_t)row] = f4(z);
                rec_next[2 * (size_t)row + 1] = f4(p);
                rr = dot3(r, r);
                rz = dot3(r, z);
            }
            rr = warp_sum(rr);
            rz = warp_sum(rz);
            if (lane == 0) {
                float* p = sm.part + (sl - first) * 3;
                p[0] = rr; p[1] = rz;
            }
        }
        auto next_iteration = [&](int s) {
            SceneState& st = sm.st[s];
            if (!st.active) return;
            const double rr = sm.tot[s * 3], rz_new = sm.tot[s * 3 + 1];
            st.iters += 1;
            st.beta = (float)(rz_new / st.rz);
            st.rz = rz_new;
            st.rr = rr;
            st.active = (rr > st.atol_sq) && (st.iters < a.maxiter);
            if (!isfinite(rr)) {
                st.active = 0;
                atomicOr(a.status, kStatusNonFinite);
            }
            if (st.active) atomicOr(&s_any, 1);
        };
        if (!reduce_across_grid(a, sm, buf1, 2, false, first, last, epoch, &s_ok, &s_any, next_iteration)) return;
    }
    } else {
    // Single-reduction (Chronopoulos-Gear) CG: one pass and one grid reduction per iteration.  Pass k
    // first applies update k with the scalars of reduction k-1 to the CTA's own rows
    //   p = u + beta p,  s = w + beta s,  x += alpha p,  r -= alpha s,
    //   u' = u - alpha (Mw + beta Ms)  (= M r'),  Ms' = Mw + beta Ms,
    // then forms w' = A u' from the neighbours' records (u' recomputed at the gather), Mw' = M w', writes
    // the row's next record (u', Mw', Ms') and the partials (r', u'), (w', u'), (r', r').  Pass 0 only
    // forms w0 = A u0 (alpha0 = gamma0 / delta0).  The convergence test of update k comes with the
    // reduction that follows its SpMV, so a converged solve has done one SpMV more than standard CG.
    for (int pass = 0; s_any; ++pass) {
        const float4* rc = (pass & 1) ? a.rec1 : a.rec0;  // (u, Mw, Ms) of this pass
        float4* rn = (pass & 1) ? a.rec0 : a.rec1;         // written for the next one
        if (a.cta_time != nullptr && threadIdx.x == 0) s_t0 = global_ns();
        if (a.tail_prefetch && a.contiguous && warp == W - 1) prefetch_last_round(a, sm, first, last, W, lane);
        for (int sl = first + warp; sl < last; sl += W) {
            const int4 sl4 = sm.slc[sl - first];
            const SceneState& st = sm.st[sl4.z & ~kResidentSlice];
            float gam = 0.f, del = 0.f, rrl = 0.f;
            if (st.active && lane < sl4.y) {
                const int row = sl4.x + lane;
                const unsigned info = sm.rinfo[(sl - first) * kSlice + lane];
                const bool prime = !st.primed;
                const float alpha = st.alpha, beta = st.beta;
                float* rs = a.resident ? res_slot(sm, sl, first, lane, a.resident, 1) : nullptr;
                const float4* own = rc + 3 * (size_t)row;
                const float4 o0 = own[0];
                float3 un, msn, r;
                if (prime) {
                    un = xyz(o0);
                    msn = f3(0.f, 0.f, 0.f);
                    r = rs ? res3(rs, 3) : xyz(a.r[row]);
                } else {
                    const float4 o1 = own[1];
                    const float o2 = reinterpret_cast<const float*>(own + 2)[0];
                    un = next_u(o0, o1, o2, alpha, beta, msn);
                    const float3 uo = xyz(o0);
                    float3 pv = rs ? res3(rs, 6) : xyz(a.p4[row]);
                    float3 sv = rs ? res3(rs, 9) : xyz(a.s4[row]);
                    const float3 wv = rs ? res3(rs, 12) : xyz(a.w4[row]);
                    float3 x = rs ? res3(rs, 0) : xyz(a.x[row]);
                    r = rs ? res3(rs, 3) : xyz(a.r[row]);
                    pv = f3(fmaf(beta, pv.x, uo.x), fmaf(beta, pv.y, uo.y), fmaf(beta, pv.z, uo.z));
                    sv = f3(fmaf(beta, sv.x, wv.x), fmaf(beta, sv.y, wv.y), fmaf(beta, sv.z, wv.z));
                    x = f3(fmaf(alpha, pv.x, x.x), fmaf(alpha, pv.y, x.y), fmaf(alpha, pv.z, x.z));
                    r = f3(fmaf(-alpha, sv.x, r.x), fmaf(-alpha, sv.y, r.y), fmaf(-alpha, sv.z, r.z));
                    if (rs) {
                        res3_store(rs, 0, x);
                        res3_store(rs, 3, r);
                        res3_store(rs, 6, pv);
                        res3_store(rs, 9, sv);
                    } else {
                        a.x[row] = f4(x);
                        a.r[row] = f4(r);
                        a.p4[row] = f4(pv);
                        a.s4[row] = f4(sv);
                    }
                }
                float3 w = un;  // fixed rows: identity (their u is zero)
                if (!(info & kFixedBit)) {
                    const int len = (int)(info & ~kFixedBit);
                    const unsigned long long pol = (sl4.z & kResidentSlice) ? pol_last : pol_first;
                    const SliceCols sc = slice_cols(sl);
                    w = prime ? row_times_u<U, CM, true>(a, sl4.w, len, lane, row, sc, rc, alpha, beta, pol)
                              : row_times_u<U, CM, false>(a, sl4.w, len, lane, row, sc, rc, alpha, beta, pol);
                }
                const float3 mw = a.resident == 2 ? res_minv_mul(rs, w, 15) : minv_mul(a.minv, row, w);
                if (rs) res3_store(rs, 12, w);
                else a.w4[row] = f4(w);
                float4* nx = rn + 3 * (size_t)row;
                nx[0] = make_float4(un.x, un.y, un.z, mw.x);
                nx[1] = make_float4(mw.y, mw.z, msn.x, msn.y);
                nx[2] = make_float4(msn.z, 0.f, 0.f, 0.f);
                gam = dot3(r, un);
                del = dot3(w, un);
                rrl = dot3(r, r);
            }
            gam = warp_sum(gam);
            del = warp_sum(del);
            rrl = warp_sum(rrl);
            if (lane == 0) {
                float* pp = sm.part + (sl - first) * 3;
                pp[0] = gam; pp[1] = del; pp[2] = rrl;
            }
        }
        if (a.cta_time != nullptr) {  // speed calibration: this CTA's pass time
            __syncthreads();
            if (threadIdx.x == 0) {
                a.cta_time[2 * blockIdx.x] += global_ns() - s_t0;
                a.cta_time[2 * blockIdx.x + 1] += 1;
            }
        }
        auto next_pass = [&](int s) {
            SceneState& st = sm.st[s];
            if (!st.active) return;
            const double gam = sm.tot[s * 3], del = sm.tot[s * 3 + 1], rr = sm.tot[s * 3 + 2];
            if (!st.primed) {  // gamma0 = r0.u0 came with the start reduction
                st.primed = 1;
                st.beta = 0.0f;
                st.alpha = (float)(st.rz / del);
                if (!isfinite(st.alpha)) {
                    st.active = 0;
                    atomicOr(a.status, kStatusNonFinite);
                }
            } else {
                st.iters += 1;
                st.rr = rr;
                st.active = (rr > st.atol_sq) && (st.iters < a.maxiter);
                if (!isfinite(rr)) {
                    st.active = 0;
                    atomicOr(a.status, kStatusNonFinite);
                }
                if (st.active) {
                    const float beta = (float)(gam / st.rz);
                    st.alpha = (float)(gam / (del - (double)beta * gam / (double)st.alpha));
                    st.beta = beta;
                    st.rz = gam;
                }
            }
            if (st.active) atomicOr(&s_any, 1);
        };
        if (!reduce_across_grid(a, sm, (pass & 1) ? buf1 : buf0, 3, false, first, last, epoch, &s_ok, &s_any,
                                next_pass))
            return;
    }
    }

    // ---------------- epilogue: restore scale, integrate, fixed restore
    for (int sl = first + warp; sl < last; sl += W) {
        const int4 sl4 = sm.slc[sl - first];
        const int2 meta = make_int2(sl4.x, sl4.y);
        if (lane >= meta.y) continue;
        const SceneState& st = sm.st[sl4.z & ~kResidentSlice];
        int row = meta.x + lane;
        float3 dv = a.resident ? res3(res_slot(sm, sl, first, lane, a.resident, V), 0) : xyz(a.x[row]);
        float sc = st.scale;
        dv = f3(dv.x / sc, dv.y / sc, dv.z / sc);
        store3(a.dv, row, dv);
        if (a.write_state) {
            bool fixed = (sm.rinfo[(sl - first) * kSlice + lane] & kFixedBit) != 0;
            float3 v = xyz(a.v4[row]) + dv;
            float3 q = xyz(a.q4[row]) + v * h;
            if (fixed) {
                q = load3(a.rest, row);
                v = f3(0.f, 0.f, 0.f);
            }
            store3(a.q_out, row, q);
            store3(a.v_out, row, v);
        }
    }
    if (blockIdx.x == 0) {
        for (int s = threadIdx.x; s < S; s += blockDim.x) {
            const SceneState& st = sm.st[s];
            SceneStats o;
            o.iterations = st.iters;
            o.rr = (float)st.rr;
            o.bb = (float)st.bb;
            o.converged = st.rr <= st.atol_sq;
            a.scene_stats[s] = o;
            a.cum_iters[s] += st.iters;
            // running max of the relative residual (non-negative floats order like their bit patterns)
            float rel = st.bb > 0.0 ? (float)sqrt(st.rr / st.bb) : 0.0f;
            if (!isfinite(rel)) rel = 1.0e30f;
            atomicMax(reinterpret_cast<int*>(a.resid_max + (a.solve_rhs != nullptr ? 1 : 0)), __float_as_int(rel));
        }
    }
}

}  // namespace

using PcgKernel = void (*)(PcgArgs);

template <int CM, int V>
PcgKernel pcg_kernel_cm(int unroll) {
    switch (unroll) {
        case 2: return pcg_kernel<2, CM, V>;
        case 4: return pcg_kernel<4, CM, V>;
        default: return pcg_kernel<1, CM, V>;
    }
}
template <int V>
PcgKernel pcg_kernel_v(int unroll, int cm) {
    return cm == 2 ? pcg_kernel_cm<2, V>(unroll) : (cm == 1 ? pcg_kernel_cm<1, V>(unroll) : pcg_kernel_cm<0, V>(unroll));
}
PcgKernel pcg_kernel_for(int unroll, int cm, int variant) {
    return variant == 1 ? pcg_kernel_v<1>(unroll, cm) : pcg_kernel_v<0>(unroll, cm);
}


cudaError_t allow_dynamic_smem(const void* kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> granted;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t& g = granted[{dev, kernel}];
    if (bytes <= g) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) g = bytes;
    return e;
}

// Grid size, slices per CTA and staging place for the handle's kernel variant
// and CTA size: as many CTAs as stay co-resident (the cooperative limit, and
// the optional cap), but no more than one per warp-count of slices.  The grid
// only shrinks from pass to pass (a smaller grid means more slices per CTA and
// possibly more shared memory), and the loop ends with a configuration whose
// occupancy covers the grid.
cudaError_t pcg_configure(Handle& h) {
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    int sms = 0, coop = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return cudaErrorNotSupported;
    const int cm = column_mode(h);
    const int V = h.cg_variant;
    PcgKernel kern = pcg_kernel_for(h.spmv_unroll, cm, V);
    // Automatic CTA size: 1024-thread CTAs once there are 8 slices per SM (fewer
    // CTAs make the grid reductions cheaper: on a 3,677-slice Tet4 system 115
    // such CTAs beat 460 of 256 threads by 8% per CG iteration); small systems
    // keep 256-thread CTAs, whose CTA barriers are cheaper than a wide CTA's.
    // Automatic CTA size.  A system of at most 32 slices (32 x 32 rows) runs as one CTA with a warp per
    // slice, so every reduction is a CTA barrier instead of a grid barrier: on the 425-node beam a CG
    // iteration is latency-bound, and the grid barrier's L2 round trips were most of it.
    const int threads = h.pcg_threads > 0 ? h.pcg_threads
                        : (h.nslices <= 32 ? std::max(64, 32 * h.nslices) : (h.nslices >= 8 * sms ? 1024 : 256));
    h.pcg_threads_used = threads;
    const int warps_per_cta = threads / 32;
    // One configuration: the grid only shrinks from pass to pass (a smaller grid
    // means more slices per CTA and possibly more shared memory), and the loop
    // ends with a layout whose occupancy covers the grid.  want_resident asks
    // for the resident row state when the staging is in shared memory.
    struct Config {
        int grid, L, stage, resident;
        size_t smem;
    };
    auto fit = [&](int want_resident, int slack_pct, Config& c) -> cudaError_t {
        int grid = (h.nslices + warps_per_cta - 1) / warps_per_cta;
        // wide CTAs on a system too small to give every SM one slice per warp:
        // one CTA per SM anyway, with fewer slices each (on 3,677 slices, 152 CTAs
        // take 16.3 us per CG iteration against 18.1 us for 115)
        if (threads == 1024 && grid < sms && h.nslices > 32) grid = std::min(sms, h.nslices);
        if (grid < 1) grid = 1;
        if (h.grid_cap > 0 && grid > h.grid_cap) grid = h.grid_cap;
        for (int pass = 0;; ++pass) {
            int L = (h.nslices + grid - 1) / grid > 0 ? (h.nslices + grid - 1) / grid : 1;
            if (slack_pct > 0) L += std::max(1, (L * slack_pct + 99) / 100);
            // the single-reduction variant hands nothing from one phase to another: no staging, and its
            // row state may be resident on its own
            bool stage = V == 0 && stage_in_smem(L, threads) && pass < 16;  // give up if it never settles
            int res = (stage || (V == 1 && pass < 16)) ? want_resident : 0;
            int per_sm = 0;
            size_t smem = 0;
            for (int attempt = 0; attempt < 3; ++attempt) {
                const SmemLayout lay = smem_layout(L, h.nscenes, stage, res, cm == 2, V);
                if ((lay.st | lay.tot | lay.segb | lay.sseg | lay.slc | lay.kmask | lay.kval | lay.rinfo | lay.stage |
                     lay.res) & 15)
                    return cudaErrorMisalignedAddress;
                if (lay.total > 227 * 1024) {
                    per_sm = 0;
                } else {
                    cudaError_t e = allow_dynamic_smem((const void*)kern, lay.total);
                    if (e != cudaSuccess) return e;
                    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, lay.total);
                    if (e != cudaSuccess) return e;
                }
                smem = lay.total;
                if (per_sm >= 1) break;
                if (res) res = 0;                // first drop the resident state,
                else if (stage) stage = false;  // then the shared staging
                else break;
            }
            if (per_sm < 1) return cudaErrorInvalidConfiguration;
            const int cap = per_sm * sms;
            if (grid <= cap) {
                c = Config{grid, L, stage ? 1 : 0, res, smem};
                return cudaSuccess;
            }
            grid = cap;
        }
    };
    Config plain{}, resident{};
    // automatic: x/r/z resident, inverse blocks from global memory (measured at least as
    // fast as keeping them resident too, with half the shared memory)
    const int want = h.resident_pref < 0 ? 1 : h.resident_pref;
    err = fit(0, 0, plain);
    if (err != cudaSuccess) return err;
    resident = plain;
    if (want > 0) {
        err = fit(want, 0, resident);
        if (err != cudaSuccess) return err;
    }
    // keep the resident state only when it costs no co-resident CTAs
    Config c = (resident.resident && resident.grid == plain.grid) ? resident : plain;
    if (h.balance && h.split_headroom > 0) {
        // room for calibrated splits to give a fast CTA more slices than the even
        // share, taken when it keeps the grid and the resident state
        Config wide{};
        err = fit(c.resident, h.split_headroom, wide);
        if (err != cudaSuccess) return err;
        if (wide.grid == c.grid && wide.resident == c.resident && wide.stage == c.stage) c = wide;
    }
    err = allow_dynamic_smem((const void*)kern, c.smem);
    if (err != cudaSuccess) return err;
    h.grid = c.grid;
    h.slices_per_cta = c.L;
    h.stage_smem = c.stage;
    h.resident = c.resident;
    h.pcg_smem = c.smem;
    return cudaSuccess;
}

cudaError_t launch_pcg(Handle& h, float dt, int write_state, float* q_out, float* v_out, float* f_ws, cudaStream_t s,
                       const float* solve_rhs, float* x_out, float tol, int maxiter, bool solve_warm) {
    PcgArgs a;
    a.valA = h.valA;
    a.valB = h.valB;
    a.valC = h.valC;
    a.scol = h.scol;
    const int cm = column_mode(h);
    a.dcol = cm > 0 ? h.dcol : nullptr;
    a.slice_kmask = h.slice_kmask;
    a.slice_kval = h.slice_kval;
    a.slice_ptr = h.slice_ptr;
    a.slice_meta = h.slice_meta;
    a.slice_scene = h.slice_scene;
    a.row_info = h.row_info;
    a.minv = h.minv;
    a.nslices = h.nslices;
    a.slices_per_cta = h.slices_per_cta;
    a.cta_slice0 = h.cta_slice0;
    a.cta_time = h.cta_time;
    a.tail_prefetch = h.tail_prefetch;
    a.cta_seg_base = h.cta_seg_base;
    a.cta_list = h.cta_list;
    a.contiguous = h.cta_contiguous;
    a.seg_start = h.seg_start;
    a.seg_pos = h.seg_pos;
    a.scene_seg0 = h.scene_seg0;
    a.nscenes = h.nscenes;
    a.seg_part = h.seg_part;
    a.nseg = h.nseg;
    a.v4 = h.v4;
    a.q4 = h.q4;
    a.rest = h.rest;
    a.spring_ptr = h.node_spring_ptr;
    a.spring_ent = h.node_spring_ent;
    a.spring_idx = h.spring_idx;
    a.spring_kd = h.spring_kd;
    a.f_ws = f_ws;
    a.dv = x_out != nullptr ? x_out : h.dv;
    a.q_out = q_out;
    a.v_out = v_out;
    a.x = h.x;
    a.r = h.r;
    a.zp0 = h.zp0;
    a.zp1 = h.zp1;
    a.stage = h.stage;
    a.stage_smem = h.stage_smem;
    a.resident = h.resident;
    a.rec0 = h.rec0;
    a.rec1 = h.rec1;
    a.p4 = h.p4;
    a.s4 = h.s4;
    a.w4 = h.w4;
    a.barrier = h.barrier;
    a.status = h.status;
    a.scene_stats = h.scene_stats;
    a.cum_iters = h.cum_iters;
    a.resid_max = h.resid_max;
    a.maxiter = maxiter >= 0 ? maxiter : h.maxiter;
    a.tol = tol > 0.0f ? tol : h.tol;
    a.dt = dt;
    a.limit_ns = h.wait_limit_ns;
    a.write_state = write_state;
    a.resident_slices = h.resident_slices;
    a.solve_rhs = solve_rhs;
    a.solve_warm = solve_warm ? 1 : 0;
    cudaError_t err = cudaMemsetAsync(h.barrier, 0, sizeof(unsigned), s);
    if (err != cudaSuccess) return err;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(h.grid);
    cfg.blockDim = dim3(h.pcg_threads_used);
    cfg.dynamicSmemBytes = h.pcg_smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, pcg_kernel_for(h.spmv_unroll, cm, h.cg_variant), a);
}

}  // namespace fem
