// fem_pcg_solve_noalloc: block-Jacobi PCG on a caller-supplied 3x3 BSR matrix
// that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc at solve time -- code
// running inside a caller-managed memory budget or a custom allocator that
// forbids runtime allocations, plugins embedded in a host application that
// owns all device memory, and real-time loops where an allocation's implicit
// device synchronisation would stall the stream.  fem_create allocates the
// handle's buffers, so those callers cannot use the handle path; this entry
// point takes the matrix, right-hand side and solution from the caller and
// keeps its own working vectors in a fixed-size static device array instead.
//
// The scratch array (kScratchBytes, enough for kMaxRows = 65,536 block rows)
// is a file-scope __device__ array: every GPU that loads this library holds it
// until the process exits.  All calls on a device share it, so calls that
// overlap on the GPU (different streams, or different host threads) race on
// it; serialise them.  Each call rewrites every scratch word it reads before
// reading it, except the grid-barrier counter, which it zeroes with a memset
// on the caller's stream before the launch.
//
// Host code cannot use the array's name as a device address, so the first
// call on each device looks the address up with cudaGetSymbolAddress (with
// that device current) and caches it, together with the launch configuration.
// Make that first call before any stream capture.  The cache is not refreshed:
// calls after cudaDeviceReset (or any teardown of the device's primary
// context) are not supported.
//
// Failures.  Every grid barrier wait is bounded (2 s, or the nanoseconds in the
// environment variable FEM_NOALLOC_WAIT_LIMIT_NS read at each call).  A CTA
// whose wait runs out, and every CTA that then sees the shared failure flag,
// skips to a common exit instead of returning, so the optional info word is
// always written: info[0] = iterations done, info[1] = status bits (1: a wait
// timed out, 2: a non-finite value in the solve).  The host zeroes info on the
// caller's stream before the launch and the kernel only ORs bits into
// info[1], so no failure report is lost.  After a non-finite value every CTA
// leaves x_inout untouched (the warm start survives); after a timeout the CTAs
// that saw it leave their rows untouched and the others may already have
// written theirs, so x_inout is unspecified.  With info == NULL neither failure
// is visible to the caller.
#include <cstdlib>
#include <mutex>

#include "fem_gb300.h"
#include "fem_math.cuh"

namespace fem {  // status reporting shared with the other entry points (fem_api.cu)
int report(int code, const char* message);
int report_cuda(cudaError_t err);
}  // namespace fem

namespace {

constexpr int kMaxRows = 65536;
constexpr int kThreads = 256;
constexpr int kMaxBlocks = 2048;
// r, z, p, y, x (3 floats each) + Minv (9 floats) per row, CTA partials, barrier
constexpr size_t kVecBytes = sizeof(float) * 3 * (size_t)kMaxRows;
constexpr size_t kScratchBytes = 5 * kVecBytes + sizeof(float) * 9 * (size_t)kMaxRows +
                                 sizeof(double) * 2 * 4 * (size_t)kMaxBlocks + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct Scratch {
    float* r;
    float* z;
    float* p;
    float* y;
    float* x;
    float* minv;
    double* part;  // [2][kMaxBlocks][4]: consecutive reductions alternate halves
    unsigned* barrier;
    int* status;
};

__host__ __device__ inline Scratch carve(unsigned char* base) {
    Scratch s;
    size_t off = 0;
    s.r = reinterpret_cast<float*>(base + off);
    off += kVecBytes;
    s.z = reinterpret_cast<float*>(base + off);
    off += kVecBytes;
    s.p = reinterpret_cast<float*>(base + off);
    off += kVecBytes;
    s.y = reinterpret_cast<float*>(base + off);
    off += kVecBytes;
    s.x = reinterpret_cast<float*>(base + off);
    off += kVecBytes;
    s.minv = reinterpret_cast<float*>(base + off);
    off += sizeof(float) * 9 * (size_t)kMaxRows;
    s.part = reinterpret_cast<double*>(base + off);
    off += sizeof(double) * 2 * 4 * (size_t)kMaxBlocks;
    s.barrier = reinterpret_cast<unsigned*>(base + off);
    s.status = reinterpret_cast<int*>(base + off + 64);
    return s;
}

struct Args {
    const int* offsets;
    const int* columns;
    const float* values;
    const float* rhs;
    float* x_inout;
    int n;
    float tol;
    int maxiter;
    int* info;  // optional device int[2]: iterations, status
    unsigned char* scratch;
    long long limit_ns;
};

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned load_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Bounded grid barrier (counter zeroed before the launch); false on timeout.
// The counter and the target are compared as a wrap-safe difference: the
// counter only grows, and no CTA runs more than one barrier ahead, so the
// difference stays far inside the signed 32-bit range however many barriers
// a solve takes.
__device__ bool barrier(const Scratch& s, unsigned& epoch, long long limit_ns, int* flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch += 1;
        const unsigned target = epoch * gridDim.x;  // modulo 2^32, like the counter
        __threadfence();
        atomicAdd(s.barrier, 1u);
        int ok = 1;
        unsigned long long t0 = now_ns();
        unsigned spins = 0;
        while ((int)(load_acquire(s.barrier) - target) < 0) {
            if ((++spins & 63u) == 1u) {
                if (atomicAdd(s.status, 0) != 0 || (long long)(now_ns() - t0) >= limit_ns) {
                    ok = 0;
                    atomicOr(s.status, 1);
                    break;
                }
            }
            __nanosleep(20);
        }
        __threadfence();
        *flag = ok;
    }
    __syncthreads();
    return *flag != 0;
}

// Deterministic grid sum: CTA partials in CTA order, every CTA gets the same
// total.  Reduction number `ph` uses half (ph & 1) of the partial array, so a
// CTA that runs ahead writes a half only after the next grid barrier, which no
// CTA passes before it has read that half's previous totals.
__device__ __forceinline__ double* half(const Scratch& s, int ph) { return s.part + (size_t)(ph & 1) * 4 * kMaxBlocks; }

__device__ void cta_partials(const Scratch& s, int ph, double v0, double v1, double v2, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        v0 += __shfl_xor_sync(0xffffffffu, v0, off);
        v1 += __shfl_xor_sync(0xffffffffu, v1, off);
        v2 += __shfl_xor_sync(0xffffffffu, v2, off);
    }
    if (lane == 0) {
        red[3 * warp] = v0;
        red[3 * warp + 1] = v1;
        red[3 * warp + 2] = v2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0;
        for (int w = 0; w < nw; ++w) {
            a += red[3 * w];
            b += red[3 * w + 1];
            c += red[3 * w + 2];
        }
        double* part = half(s, ph);
        part[4 * blockIdx.x] = a;
        part[4 * blockIdx.x + 1] = b;
        part[4 * blockIdx.x + 2] = c;
    }
}

__device__ void grid_totals(const Scratch& s, int ph, double* tot) {
    if (threadIdx.x == 0) {
        const double* part = half(s, ph);
        double a = 0, b = 0, c = 0;
        for (int k = 0; k < (int)gridDim.x; ++k) {
            a += part[4 * k];
            b += part[4 * k + 1];
            c += part[4 * k + 2];
        }
        tot[0] = a;
        tot[1] = b;
        tot[2] = c;
    }
    __syncthreads();
}

__device__ __forceinline__ void row_mul(const Args& a, const float* vec, int i, float* out) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int k = a.offsets[i]; k < a.offsets[i + 1]; ++k) {
        const float* b = a.values + 9 * (size_t)k;
        const float* p = vec + 3 * (size_t)a.columns[k];
        s0 += b[0] * p[0] + b[1] * p[1] + b[2] * p[2];
        s1 += b[3] * p[0] + b[4] * p[1] + b[5] * p[2];
        s2 += b[6] * p[0] + b[7] * p[1] + b[8] * p[2];
    }
    out[0] = s0;
    out[1] = s1;
    out[2] = s2;
}

// The solve proper.  Returns the CG iterations done and sets *fail: bit 1 when
// a barrier wait ran out (this CTA's or, seen through the shared status word,
// another CTA's), bit 2 when a grid total is non-finite (every CTA forms the
// same totals, so every CTA sets it at the same point).  Either way the CTA
// goes straight to the common exit.
__device__ int noalloc_solve(const Args& a, const Scratch& s, double* red, double* tot, int* flag, float* scale_out,
                             int* fail) {
    const int n = a.n;
    const int rows_per_cta = (n + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * rows_per_cta;
    const int r1 = min(n, r0 + rows_per_cta);
    unsigned epoch = 0;
    int ph = 0;  // reduction counter (selects the partial-array half)
    *fail = 0;
    *scale_out = 1.0f;

    // preconditioner from the diagonal blocks (identity where a row has none), max |b|
    double mx = 0.0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        float d[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
        for (int k = a.offsets[i]; k < a.offsets[i + 1]; ++k)
            if (a.columns[k] == i)
                for (int c = 0; c < 9; ++c) d[c] = a.values[9 * (size_t)k + c];
        fem::inverse_diagonal_block(d, s.minv + 9 * (size_t)i);
        for (int c = 0; c < 3; ++c) mx = fmax(mx, (double)fabsf(a.rhs[3 * (size_t)i + c]));
    }
    // max over the grid via the same partial slots (max of non-negatives, fixed order)
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        if (lane == 0) red[warp] = mx;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
            half(s, ph)[4 * blockIdx.x + 3] = m;
        }
    }
    if (!barrier(s, epoch, a.limit_ns, flag)) {
        *fail = 1;
        return 0;
    }
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int k = 0; k < (int)gridDim.x; ++k) m = fmax(m, half(s, ph)[4 * k + 3]);
        tot[0] = m;
    }
    __syncthreads();
    ++ph;
    const float maximum = (float)tot[0];
    const float scale = (maximum > 0.0f && maximum < 1.0e-12f) ? fminf(1.0f / maximum, 1.0e30f) : 1.0f;
    *scale_out = scale;
    __syncthreads();

    // x0 = scaled warm start (zero when b == 0)
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x)
        for (int c = 0; c < 3; ++c)
            s.x[3 * (size_t)i + c] = maximum == 0.0f ? 0.0f : scale * a.x_inout[3 * (size_t)i + c];
    if (!barrier(s, epoch, a.limit_ns, flag)) {
        *fail = 1;
        return 0;
    }
    double rr = 0, rz = 0, bb = 0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        float ax[3];
        row_mul(a, s.x, i, ax);
        float r[3], z[3];
        for (int c = 0; c < 3; ++c) {
            float b = scale * a.rhs[3 * (size_t)i + c];
            r[c] = b - ax[c];
            bb += (double)b * b;
        }
        const float* m = s.minv + 9 * (size_t)i;
        for (int c = 0; c < 3; ++c) z[c] = m[3 * c] * r[0] + m[3 * c + 1] * r[1] + m[3 * c + 2] * r[2];
        for (int c = 0; c < 3; ++c) {
            s.r[3 * (size_t)i + c] = r[c];
            s.z[3 * (size_t)i + c] = z[c];
            s.p[3 * (size_t)i + c] = z[c];
            rr += (double)r[c] * r[c];
            rz += (double)r[c] * z[c];
        }
    }
    cta_partials(s, ph, rr, rz, bb, red);
    if (!barrier(s, epoch, a.limit_ns, flag)) {
        *fail = 1;
        return 0;
    }
    grid_totals(s, ph++, tot);
    rr = tot[0];
    rz = tot[1];
    bb = tot[2];
    const double atol_sq = (double)a.tol * a.tol * bb;
    int it = 0;
    if (!isfinite(rr)) {  // every CTA sees the same totals, so all of them stop here
        *fail = 2;
        return it;
    }
    while (it < a.maxiter && rr > atol_sq) {
        double pap = 0;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            float y[3];
            row_mul(a, s.p, i, y);
            for (int c = 0; c < 3; ++c) {
                s.y[3 * (size_t)i + c] = y[c];
                pap += (double)s.p[3 * (size_t)i + c] * y[c];
            }
        }
        cta_partials(s, ph, pap, 0.0, 0.0, red);
        if (!barrier(s, epoch, a.limit_ns, flag)) {
            *fail = 1;
            return it;
        }
        grid_totals(s, ph++, tot);
        const float alpha = (float)(rz / tot[0]);
        __syncthreads();
        if (!isfinite(alpha)) {  // same value in every CTA: all stop before touching x
            *fail = 2;
            return it;
        }
        double rr_l = 0, rz_l = 0;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            float r[3];
            for (int c = 0; c < 3; ++c) {
                size_t k = 3 * (size_t)i + c;
                s.x[k] += alpha * s.p[k];
                r[c] = s.r[k] - alpha * s.y[k];
                s.r[k] = r[c];
            }
            const float* m = s.minv + 9 * (size_t)i;
            for (int c = 0; c < 3; ++c) {
                float z = m[3 * c] * r[0] + m[3 * c + 1] * r[1] + m[3 * c + 2] * r[2];
                s.z[3 * (size_t)i + c] = z;
                rr_l += (double)r[c] * r[c];
                rz_l += (double)r[c] * z;
            }
        }
        cta_partials(s, ph, rr_l, rz_l, 0.0, red);
        if (!barrier(s, epoch, a.limit_ns, flag)) {
            *fail = 1;
            return it;
        }
        grid_totals(s, ph++, tot);
        const float beta = (float)(tot[1] / rz);
        rr = tot[0];
        rz = tot[1];
        __syncthreads();
        ++it;
        if (!isfinite(rr)) {
            *fail = 2;
            return it;
        }
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x)
            for (int c = 0; c < 3; ++c) {
                size_t k = 3 * (size_t)i + c;
                s.p[k] = s.z[k] + beta * s.p[k];
            }
        if (!barrier(s, epoch, a.limit_ns, flag)) {
            *fail = 1;
            return it;
        }
    }
    return it;
}

__global__ void __launch_bounds__(kThreads) noalloc_pcg_kernel(Args a) {
    __shared__ double red[3 * 32];
    __shared__ double tot[3];
    __shared__ int flag;
    const Scratch s = carve(a.scratch);
    float scale = 1.0f;
    int fail = 0;
    const int it = noalloc_solve(a, s, red, tot, &flag, &scale, &fail);
    // Common exit.  A CTA that saw a failure keeps the caller's warm start in
    // its rows of x_inout and ORs the failure into info[1] (zeroed by the host).
    if (fail == 0) {
        const int n = a.n;
        const int rows_per_cta = (n + gridDim.x - 1) / gridDim.x;
        const int r0 = blockIdx.x * rows_per_cta;
        const int r1 = min(n, r0 + rows_per_cta);
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x)
            for (int c = 0; c < 3; ++c) a.x_inout[3 * (size_t)i + c] = s.x[3 * (size_t)i + c] / scale;
    }
    if (threadIdx.x == 0 && a.info != nullptr) {
        if (fail != 0) atomicOr(a.info + 1, fail);
        if (blockIdx.x == 0) a.info[0] = it;
    }
}

struct DeviceSetup {
    bool ready = false;
    unsigned char* scratch = nullptr;
    int max_grid = 0;
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[64];

// Once per device, with that device current: resolve the scratch array's
// device address and the cooperative grid limit.
int setup_device(DeviceSetup** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return fem::report(FEM_ERR_CUDA, "fem_pcg_solve_noalloc: no current CUDA device");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup& d = g_setup[dev];
    if (!d.ready) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || ptr == nullptr)
            return fem::report(FEM_ERR_CUDA, "fem_pcg_solve_noalloc: scratch symbol unavailable");
        int sms = 0, coop = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return fem::report(FEM_ERR_CUDA, "fem_pcg_solve_noalloc: device query failed");
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
            return fem::report(FEM_ERR_UNSUPPORTED, "fem_pcg_solve_noalloc: cooperative launch unavailable");
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, noalloc_pcg_kernel, kThreads, 0) != cudaSuccess ||
            per_sm < 1)
            return fem::report(FEM_ERR_CUDA, "fem_pcg_solve_noalloc: occupancy query failed");
        d.scratch = static_cast<unsigned char*>(ptr);
        d.max_grid = per_sm * sms < kMaxBlocks ? per_sm * sms : kMaxBlocks;
        d.ready = true;
    }
    *out = &d;
    return FEM_OK;
}

}  // namespace

extern "C" int fem_pcg_solve_noalloc(const int32_t* offsets, const int32_t* columns, const float* values,
                                     const float* rhs, float* x_inout, int32_t rows, float tolerance,
                                     int32_t maxiter, int32_t* info, void* stream) {
    if (rows < 0 || rows > kMaxRows)  // beyond the static scratch capacity
        return fem::report(FEM_ERR_BAD_ARG, "fem_pcg_solve_noalloc: rows outside [0, 65536]");
    if (!(tolerance > 0.0f) || maxiter < 0)
        return fem::report(FEM_ERR_BAD_ARG, "fem_pcg_solve_noalloc: tolerance must be positive and maxiter non-negative");
    if (rows == 0) return FEM_OK;
    if (!offsets || !columns || !values || !rhs || !x_inout)
        return fem::report(FEM_ERR_BAD_ARG, "fem_pcg_solve_noalloc: null argument");
    DeviceSetup* d = nullptr;
    int code = setup_device(&d);
    if (code != FEM_OK) return code;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Scratch sc = carve(d->scratch);
    if (cudaError_t e = cudaMemsetAsync(sc.barrier, 0, 128, s); e != cudaSuccess)  // barrier + status
        return fem::report_cuda(e);
    if (info != nullptr)  // the kernel ORs failure bits into info[1]
        if (cudaError_t e = cudaMemsetAsync(info, 0, 2 * sizeof(int32_t), s); e != cudaSuccess)
            return fem::report_cuda(e);
    long long limit_ns = 2000000000LL;
    if (const char* env = std::getenv("FEM_NOALLOC_WAIT_LIMIT_NS")) {
        char* end = nullptr;
        const long long v = std::strtoll(env, &end, 10);
        if (end == env || *end != '\0' || v < 0)
            return fem::report(FEM_ERR_BAD_ARG, "fem_pcg_solve_noalloc: FEM_NOALLOC_WAIT_LIMIT_NS must be a "
                                                "non-negative integer");
        limit_ns = v;
    }
    int rows_per_cta_min = 64;  // keep CTAs busy
    int grid = (rows + rows_per_cta_min - 1) / rows_per_cta_min;
    if (grid > d->max_grid) grid = d->max_grid;
    if (grid < 1) grid = 1;
    Args a;
    a.offsets = offsets;
    a.columns = columns;
    a.values = values;
    a.rhs = rhs;
    a.x_inout = x_inout;
    a.n = rows;
    a.tol = tolerance;
    a.maxiter = maxiter;
    a.info = info;
    a.scratch = d->scratch;
    a.limit_ns = limit_ns;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return fem::report_cuda(cudaLaunchKernelEx(&cfg, noalloc_pcg_kernel, a));
}
