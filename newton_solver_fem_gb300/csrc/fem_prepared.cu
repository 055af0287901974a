// Prepared affine step: the reference's PreparedFEMStep (prepared_step.py:64-302)
// over the handle's assembled matrix.
//
//   fem_prepare              copy q, v (fixed nodes restored in the copy), evaluate the
//                            force terms once: impulse = h sum f (+ h ext), predictor
//                            sum_j A_ij (v_j - v_i), diagonal blocks of PAP + I - P and
//                            base_rhs = rhs(no extra load)              (lines 126-183)
//   fem_prepared_rhs         impulse + h ext - predictor + spring damping, projected
//                                                                        (lines 185-213)
//   fem_apply_operator       (PAP + I - P) x                             (lines 215-224)
//   fem_apply_preconditioner block-Jacobi M r                            (lines 226-235)
//   fem_prepared_solve       normalised PCG from the workspace's increment (lines 252-275)
//   fem_prepared_reconstruct v' = v + dv, q' = q + h v', fixed restored   (lines 277-302)
//
// The workspace arrays belong to the caller (FemPreparedWs), so every entry
// point is stateless with respect to it and the pointers stay stable for
// CUDA graphs.
#include "fem_internal.cuh"
#include "fem_math.cuh"

namespace fem {
namespace {

__device__ __forceinline__ float3 ld3(const float* p, int i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void st3(float* p, int i, float3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
__device__ __forceinline__ float3 block_mul(float4 a, float4 b, float c, float3 p) {
    return f3(a.x * p.x + a.y * p.y + a.z * p.z, a.w * p.x + b.x * p.y + b.y * p.z, b.z * p.x + b.w * p.y + c * p.z);
}

// Workspace state: fixed nodes take their rest position and zero velocity
// (fixed_particles.py:11-21), applied to the copy only.
__global__ void prepare_state_kernel(int P, const float* __restrict__ q_in, const float* __restrict__ v_in,
                                     const unsigned char* __restrict__ fixed, const float* __restrict__ rest,
                                     float* __restrict__ pq, float* __restrict__ pv, float4* __restrict__ q4,
                                     float4* __restrict__ v4) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const bool fx = fixed[i] != 0;
    const float3 q = fx ? ld3(rest, i) : ld3(q_in, i);
    const float3 v = fx ? f3(0.f, 0.f, 0.f) : ld3(v_in, i);
    st3(pq, i, q);
    st3(pv, i, v);
    q4[i] = f4(q);
    v4[i] = f4(v);
}

// One warp per SELL slice, lane per row: predictor sum_k A_ik (v_k - v_i) and
// the diagonal block of PAP + I - P (A_ii, identity at fixed rows).
__global__ void predictor_diag_kernel(int nslices, const int* __restrict__ slice_ptr, const int2* __restrict__ meta,
                                      const unsigned* __restrict__ row_info, const float4* __restrict__ valA,
                                      const float4* __restrict__ valB, const float* __restrict__ valC,
                                      const int* __restrict__ scol, const float4* __restrict__ v4,
                                      float* __restrict__ pred, float* __restrict__ diag) {
    const int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (sl >= nslices) return;
    const int2 m = meta[sl];
    if (lane >= m.y) return;
    const int row = m.x + lane;
    const unsigned info = row_info[row];
    const int len = (int)(info & ~kFixedBit);
    const float3 vi = xyz(v4[row]);
    float3 acc = f3(0.f, 0.f, 0.f);
    float d[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < len; ++k) {
        const size_t e = (size_t)(slice_ptr[sl] + k) * kSlice + lane;
        const float4 a = valA[e], b = valB[e];
        const float c = valC[e];
        const int j = scol[e];
        acc = acc + block_mul(a, b, c, xyz(v4[j]) - vi);
        if (j == row) {
            d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
            d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = b.w; d[8] = c;
        }
    }
    if (info & kFixedBit) {
        for (int k = 0; k < 9; ++k) d[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    }
    st3(pred, row, acc);
    for (int k = 0; k < 9; ++k) diag[9 * (size_t)row + k] = d[k];
}

// out = impulse + h ext - predictor, then the spring damping restore
// (implicit_predictor.py:28-41), then zero at fixed rows (fixed_particles.py:159-160).
__global__ void prepared_rhs_kernel(int P, const float* __restrict__ impulse, const float* __restrict__ ext, float dt,
                                    const float* __restrict__ pred, const int* __restrict__ sptr,
                                    const int* __restrict__ sent, const int* __restrict__ sidx,
                                    const float* __restrict__ skd, const float* __restrict__ pv,
                                    const unsigned char* __restrict__ fixed, float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    if (fixed[i]) {
        st3(out, i, f3(0.f, 0.f, 0.f));
        return;
    }
    float3 r = ld3(impulse, i);
    if (ext != nullptr) r = r + ld3(ext, i) * dt;
    r = r - ld3(pred, i);
    for (int e = sptr[i]; e < sptr[i + 1]; ++e) {
        const int ent = sent[e], s = ent >> 1;
        const int ia = sidx[2 * s], ib = sidx[2 * s + 1];
        if (ia < 0 || ib < 0) continue;
        const float3 corr = (ld3(pv, ia) - ld3(pv, ib)) * (dt * skd[s]);
        r = (ent & 1) ? r - corr : r + corr;
    }
    st3(out, i, r);
}

// y = (PAP + I - P) x (fixed_particles.py:56-73): fixed rows return x_i, free
// rows skip fixed columns and sum in k order.  One warp per SELL slice and lane
// per row, streamed like the PCG's SpMV: kOperatorBatch block columns loaded
// before any is used, the column as a 16-bit offset when the handle has them,
// the blocks through the non-coherent path without L1 allocation, and the
// fixed columns read from a per-(slice, k) lane mask rather than from each
// column's row info.
// kOperatorBatch block columns in flight per thread (FEM_TUNE_OPERATOR_BATCH): 2 at 32 registers (eight
// 256-thread CTAs, 64 warps per SM) holds a 64^3 Hex8 matrix's 8,582 slices in one wave on 152 SMs and
// streams it in 51 us (0.82 of the measured copy bandwidth); 4 at 48 registers (five CTAs per SM) needs
// 1.4 waves, and its half-empty second wave takes it to 63 us.
__device__ __forceinline__ float4 ld_stream4(const float4* p) {
    float4 v;
    asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ float ld_stream1(const float* p) {
    float v;
    asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
template <int kOperatorBatch>
__global__ void __launch_bounds__(256, kOperatorBatch == 2 ? 8 : 5) apply_operator_kernel(
    int nslices, const int* __restrict__ slice_ptr, const int2* __restrict__ meta,
    const unsigned* __restrict__ row_info, const float4* __restrict__ valA, const float4* __restrict__ valB,
    const float* __restrict__ valC, const int* __restrict__ scol, const short* __restrict__ dcol,
    const unsigned* __restrict__ fixcol, const float* __restrict__ x, float* __restrict__ y) {
    const int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (sl >= nslices) return;
    const int2 m = meta[sl];
    if (lane >= m.y) return;
    const int row = m.x + lane;
    const unsigned info = row_info[row];
    if (info & kFixedBit) {
        st3(y, row, ld3(x, row));
        return;
    }
    const int len = (int)(info & ~kFixedBit), base = slice_ptr[sl];
    float3 acc = f3(0.f, 0.f, 0.f);
    for (int k0 = 0; k0 < len; k0 += kOperatorBatch) {
        float4 A[kOperatorBatch], B[kOperatorBatch];
        float C[kOperatorBatch];
        int j[kOperatorBatch];
        bool use[kOperatorBatch];
#pragma unroll
        for (int u = 0; u < kOperatorBatch; ++u) {
            const int k = k0 + u < len ? k0 + u : len - 1;  // a repeated last column is loaded, not added
            const size_t e = (size_t)(base + k) * kSlice + lane;
            A[u] = ld_stream4(valA + e);
            B[u] = ld_stream4(valB + e);
            C[u] = ld_stream1(valC + e);
            j[u] = dcol != nullptr ? row + (int)__ldg(dcol + e) : __ldg(scol + e);
            use[u] = k0 + u < len && (fixcol == nullptr || ((__ldg(fixcol + base + k) >> lane) & 1u) == 0u);
        }
        float3 xj[kOperatorBatch];
#pragma unroll
        for (int u = 0; u < kOperatorBatch; ++u) xj[u] = ld3(x, j[u]);
#pragma unroll
        for (int u = 0; u < kOperatorBatch; ++u)
            if (use[u]) acc = acc + block_mul(A[u], B[u], C[u], xj[u]);
    }
    st3(y, row, acc);
}

// The same product with the block planes staged through shared memory by bulk asynchronous copies
// (cp.async.bulk, completing on an mbarrier): lane 0 of each warp copies kCols block columns of its
// slice (values and 16-bit column offsets: 38 B per block, contiguous per plane in the SELL layout)
// into one half of the warp's double buffer while the warp computes from the other half.  Waits
// are bounded by limit_ns; on a timeout the kernel sets the timeout status, waits (again bounded)
// for the copies it issued and returns.  Same arithmetic in the same order as the direct kernel.
constexpr int kStageWarps = 4;
template <int kCols>
struct StageLayout {
    static constexpr int a = 0, b = kCols * kSlice * 16, c = 2 * kCols * kSlice * 16, d = c + kCols * kSlice * 4;
    static constexpr int bytes = d + kCols * kSlice * 2;  // per buffer
    static constexpr int total = kStageWarps * 2 * bytes + kStageWarps * 2 * 8;  // buffers, then mbarriers
    static_assert(b % 16 == 0 && c % 16 == 0 && d % 16 == 0 && bytes % 16 == 0, "16-byte bulk copy targets");
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait of a whole warp for phase `parity` of `bar`: every lane observes the phase (so the
// copied bytes are visible to it), and the timeout decision is the same in every lane (lane 0's
// clock).  False after limit_ns.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, long long limit_ns) {
    bool done = mbar_try_wait(bar, parity);
    if (__all_sync(0xffffffffu, done)) return true;
    const unsigned long long t0 = __shfl_sync(0xffffffffu, global_ns(), 0);
    for (;;) {
        if (!done) done = mbar_try_wait(bar, parity);
        if (__all_sync(0xffffffffu, done)) return true;
        const unsigned long long t = __shfl_sync(0xffffffffu, global_ns(), 0);
        if ((long long)(t - t0) >= limit_ns) return false;
    }
}
// Bounded wait of one thread (the timeout path's drain of copies still in flight).
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity, long long limit_ns) {
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity) && (long long)(global_ns() - t0) < limit_ns) {
    }
}

template <int kCols>
__global__ void __launch_bounds__(kStageWarps * 32) apply_operator_staged_kernel(
    int nslices, const int* __restrict__ slice_ptr, const int2* __restrict__ meta,
    const unsigned* __restrict__ row_info, const float4* __restrict__ valA, const float4* __restrict__ valB,
    const float* __restrict__ valC, const short* __restrict__ dcol, const unsigned* __restrict__ fixcol,
    const float* __restrict__ x, float* __restrict__ y, int* __restrict__ status, long long limit_ns) {
    using L = StageLayout<kCols>;
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sl = blockIdx.x * kStageWarps + w;
    if (sl >= nslices) return;  // the whole warp: nothing below synchronises across warps
    unsigned char* buf = smem + (size_t)w * 2 * L::bytes;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + (size_t)kStageWarps * 2 * L::bytes) + 2 * w;
    const int base = slice_ptr[sl], len_slice = slice_ptr[sl + 1] - base;
    const int nchunks = (len_slice + kCols - 1) / kCols;
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar + 1)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    auto issue = [&](int c) {  // lane 0: chunk c into buffer c & 1
        const int k0 = c * kCols, nk = min(kCols, len_slice - k0);
        const size_t e0 = (size_t)(base + k0) * kSlice;
        unsigned char* dst = buf + (size_t)(c & 1) * L::bytes;
        uint64_t* b = bar + (c & 1);
        const uint32_t tx = (uint32_t)nk * kSlice * (16 + 16 + 4 + 2);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier reads of this buffer first
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(tx)
                     : "memory");
        bulk_g2s(dst + L::a, valA + e0, (uint32_t)nk * kSlice * 16, b);
        bulk_g2s(dst + L::b, valB + e0, (uint32_t)nk * kSlice * 16, b);
        bulk_g2s(dst + L::c, valC + e0, (uint32_t)nk * kSlice * 4, b);
        bulk_g2s(dst + L::d, dcol + e0, (uint32_t)nk * kSlice * 2, b);
    };
    if (lane == 0) {
        issue(0);
        if (nchunks > 1) issue(1);
    }
    const int2 m = meta[sl];
    const int row = m.x + lane;
    const bool valid = lane < m.y;
    const unsigned info = valid ? row_info[row] : 0u;
    const bool fixed = valid && (info & kFixedBit) != 0;
    const int len = valid ? (int)(info & ~kFixedBit) : 0;
    float3 acc = f3(0.f, 0.f, 0.f);
    int failed = -1;  // the chunk whose wait ran out (chunks failed and failed + 1 may be in flight)
    for (int c = 0; c < nchunks; ++c) {
        if (!mbar_wait_warp(bar + (c & 1), (uint32_t)((c >> 1) & 1), limit_ns)) {
            failed = c;
            break;
        }
        const unsigned char* src = buf + (size_t)(c & 1) * L::bytes;
        const float4* sA = reinterpret_cast<const float4*>(src + L::a);
        const float4* sB = reinterpret_cast<const float4*>(src + L::b);
        const float* sC = reinterpret_cast<const float*>(src + L::c);
        const short* sD = reinterpret_cast<const short*>(src + L::d);
        const int k0 = c * kCols, nk = min(kCols, len_slice - k0);
#pragma unroll
        for (int kk = 0; kk < kCols; ++kk) {
            const int k = k0 + kk;
            if (kk < nk && !fixed && k < len) {
                const int i = kk * kSlice + lane;
                const bool use = fixcol == nullptr || ((__ldg(fixcol + base + k) >> lane) & 1u) == 0u;
                const float3 xj = ld3(x, row + (int)sD[i]);
                if (use) acc = acc + block_mul(sA[i], sB[i], sC[i], xj);
            }
        }
        __syncwarp();  // every lane is done with this buffer before it is refilled
        if (lane == 0 && c + 2 < nchunks) issue(c + 2);
    }
    if (failed >= 0) {  // warp-uniform
        if (lane == 0) {
            atomicOr(status, kStatusTimeout);
            // the copies of chunks failed and failed + 1 were issued and may still be landing
            for (int c = failed; c < nchunks && c <= failed + 1; ++c)
                mbar_drain(bar + (c & 1), (uint32_t)((c >> 1) & 1), limit_ns);
        }
        __syncwarp();
        return;
    }
    if (!valid) return;
    if (fixed) {
        st3(y, row, ld3(x, row));
        return;
    }
    st3(y, row, acc);
}

__global__ void apply_preconditioner_kernel(int P, const float* __restrict__ minv, const float* __restrict__ r,
                                            float* __restrict__ z) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const float* b = minv + 9 * (size_t)i;
    const float3 v = ld3(r, i);
    st3(z, i, f3(b[0] * v.x + b[1] * v.y + b[2] * v.z, b[3] * v.x + b[4] * v.y + b[5] * v.z,
                 b[6] * v.x + b[7] * v.y + b[8] * v.z));
}

__global__ void pack_warm_start_kernel(int P, const float* __restrict__ dv, const unsigned char* __restrict__ fixed,
                                       float4* __restrict__ x4) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    x4[i] = fixed[i] ? make_float4(0.f, 0.f, 0.f, 0.f) : f4(ld3(dv, i));
}

// kernels.py:115-128 (update_state), then the fixed restore.
__global__ void reconstruct_kernel(int P, const float* __restrict__ dv, const float* __restrict__ pq,
                                   const float* __restrict__ pv, const unsigned char* __restrict__ fixed,
                                   const float* __restrict__ rest, float dt, float* __restrict__ q_out,
                                   float* __restrict__ v_out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float3 v = ld3(pv, i) + ld3(dv, i);
    float3 q = ld3(pq, i) + v * dt;
    if (fixed[i]) {
        q = ld3(rest, i);
        v = f3(0.f, 0.f, 0.f);
    }
    st3(q_out, i, q);
    st3(v_out, i, v);
}

inline int blocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

bool ws_ok(const FemPreparedWs* w) {
    return w && w->q && w->v && w->impulse && w->predictor && w->base_rhs && w->increment && w->diagonal;
}

struct Guard {
    int prev = -1;
    explicit Guard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~Guard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};


cudaError_t launch_rhs(Handle& h, const FemPreparedWs* w, const float* ext, float dt, float* out, cudaStream_t s) {
    prepared_rhs_kernel<<<blocks(h.P, 256), 256, 0, s>>>(h.P, w->impulse, ext, dt, w->predictor, h.node_spring_ptr,
                                                         h.node_spring_ent, h.spring_idx, h.spring_kd, w->v,
                                                         h.fixed_mask, out);
    return cudaGetLastError();
}

}  // namespace
}  // namespace fem

using fem::Handle;

extern "C" {

int fem_prepare(FemHandle* H, const FemPreparedWs* w, const float* q_in, const float* v_in,
                const float* external_forces, const float* activations, const float* gravity, float dt,
                void* stream) {
    if (H == nullptr || !fem::ws_ok(w) || q_in == nullptr || v_in == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_prepare: null handle, workspace array or state");
    Handle& h = H->h;
    if (!(dt > 0.0f)) return fem::report(FEM_ERR_BAD_ARG, "fem_prepare: dt must be positive");
    if (h.enable_act && h.T > 0 && activations == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_prepare: tet activations are enabled but none were passed");
    if (h.P == 0) return FEM_OK;
    fem::Guard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    fem::prepare_state_kernel<<<fem::blocks(h.P, 256), 256, 0, s>>>(h.P, q_in, v_in, h.fixed_mask, h.rest, w->q,
                                                                      w->v, h.q4, h.v4);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = fem::launch_element_forces(h, activations, s);
    if (err == cudaSuccess)
        err = fem::launch_node_forces(h, external_forces, gravity, dt, FEM_TERM_ALL, true, w->impulse, s);
    if (err == cudaSuccess && h.nslices > 0) {
        fem::predictor_diag_kernel<<<fem::blocks((int64_t)h.nslices * 32, 256), 256, 0, s>>>(
            h.nslices, h.slice_ptr, h.slice_meta, h.row_info, h.valA, h.valB, h.valC, h.scol, h.v4, w->predictor,
            w->diagonal);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = fem::launch_rhs(h, w, nullptr, dt, w->base_rhs, s);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(w->increment, h.dv, sizeof(float) * 3 * (size_t)h.P, cudaMemcpyDeviceToDevice, s);
    return fem::report_cuda(err);
}

int fem_prepared_rhs(FemHandle* H, const FemPreparedWs* w, const float* external_forces, float dt, float* out,
                     void* stream) {
    if (H == nullptr || !fem::ws_ok(w) || out == nullptr || out == external_forces)
        return fem::report(FEM_ERR_BAD_ARG, "fem_prepared_rhs: null argument or output aliasing the load");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    fem::Guard g(H->device);
    return fem::report_cuda(fem::launch_rhs(h, w, external_forces, dt, out, (cudaStream_t)stream));
}

int fem_apply_operator(FemHandle* H, const float* x, float* y, void* stream) {
    if (H == nullptr || x == nullptr || y == nullptr || x == y)
        return fem::report(FEM_ERR_BAD_ARG, "fem_apply_operator: null or aliased vectors");
    Handle& h = H->h;
    if (h.P == 0 || h.nslices == 0) return FEM_OK;
    fem::Guard g(H->device);
    if (h.operator_stage != 0 && h.dcol != nullptr) {
        const int grid = (h.nslices + fem::kStageWarps - 1) / fem::kStageWarps;
        cudaError_t err;
        if (h.operator_stage == 4) {
            using L = fem::StageLayout<4>;
            err = fem::allow_dynamic_smem((const void*)fem::apply_operator_staged_kernel<4>, L::total);
            if (err == cudaSuccess)
                fem::apply_operator_staged_kernel<4><<<grid, fem::kStageWarps * 32, L::total, (cudaStream_t)stream>>>(
                    h.nslices, h.slice_ptr, h.slice_meta, h.row_info, h.valA, h.valB, h.valC, h.dcol, h.fixcol, x, y,
                    h.status, h.wait_limit_ns);
        } else {
            using L = fem::StageLayout<8>;
            err = fem::allow_dynamic_smem((const void*)fem::apply_operator_staged_kernel<8>, L::total);
            if (err == cudaSuccess)
                fem::apply_operator_staged_kernel<8><<<grid, fem::kStageWarps * 32, L::total, (cudaStream_t)stream>>>(
                    h.nslices, h.slice_ptr, h.slice_meta, h.row_info, h.valA, h.valB, h.valC, h.dcol, h.fixcol, x, y,
                    h.status, h.wait_limit_ns);
        }
        if (err != cudaSuccess) return fem::report_cuda(err);
        return fem::report_cuda(cudaGetLastError());
    }
    auto kern = h.operator_batch == 2 ? fem::apply_operator_kernel<2> : fem::apply_operator_kernel<4>;
    kern<<<fem::blocks((int64_t)h.nslices * 32, 256), 256, 0, (cudaStream_t)stream>>>(
        h.nslices, h.slice_ptr, h.slice_meta, h.row_info, h.valA, h.valB, h.valC, h.scol, h.dcol, h.fixcol, x, y);
    return fem::report_cuda(cudaGetLastError());
}

int fem_apply_preconditioner(FemHandle* H, const float* r, float* z, void* stream) {
    if (H == nullptr || r == nullptr || z == nullptr || r == z)
        return fem::report(FEM_ERR_BAD_ARG, "fem_apply_preconditioner: null or aliased vectors");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    fem::Guard g(H->device);
    fem::apply_preconditioner_kernel<<<fem::blocks(h.P, 256), 256, 0, (cudaStream_t)stream>>>(h.P, h.minv, r, z);
    return fem::report_cuda(cudaGetLastError());
}

int fem_prepared_solve(FemHandle* H, const FemPreparedWs* w, const float* rhs, float tolerance, int32_t maxiter,
                       float dt, void* stream) {
    if (H == nullptr || !fem::ws_ok(w) || rhs == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_prepared_solve: null handle, workspace array or rhs");
    if (!(tolerance > 0.0f) || maxiter < 0)
        return fem::report(FEM_ERR_BAD_ARG, "fem_prepared_solve: tolerance must be positive and maxiter non-negative");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    fem::Guard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    fem::pack_warm_start_kernel<<<fem::blocks(h.P, 256), 256, 0, s>>>(h.P, w->increment, h.fixed_mask, h.x);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess)
        err = fem::launch_pcg(h, dt, 0, nullptr, nullptr, nullptr, s, rhs, w->increment, tolerance, maxiter,
                              /*solve_warm=*/true);
    return fem::report_cuda(err);
}

int fem_prepared_reconstruct(FemHandle* H, const FemPreparedWs* w, const float* dv, float dt, float* q_out,
                             float* v_out, void* stream) {
    if (H == nullptr || !fem::ws_ok(w) || dv == nullptr || q_out == nullptr || v_out == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_prepared_reconstruct: null argument");
    if (q_out == w->q || v_out == w->v)
        return fem::report(FEM_ERR_BAD_ARG, "fem_prepared_reconstruct: outputs must not be the prepared state");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    fem::Guard g(H->device);
    fem::reconstruct_kernel<<<fem::blocks(h.P, 256), 256, 0, (cudaStream_t)stream>>>(
        h.P, dv, w->q, w->v, h.fixed_mask, h.rest, dt, q_out, v_out);
    return fem::report_cuda(cudaGetLastError());
}

}  // extern "C"
