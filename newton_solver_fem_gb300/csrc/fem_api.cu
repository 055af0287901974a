// C ABI of libfemgb300.so: handle construction (pattern, SELL layout,
// incidence lists, launch configuration) and the per-substep entry points.
// Host-side setup replaces SolverFEM.__init__ (solver.py:212-415) and Warp's
// bsr_set_from_triplets / map_triplet_blocks (solver.py:331-337, 823-846;
// sparse_update.py:9-30): the sparsity pattern is the set of valid triplet
// (row, col) pairs of the reference layout, columns sorted per row, and each
// slot keeps its contributing triplets in ascending order.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "fem_internal.cuh"

namespace fem {
}  // namespace fem

namespace {

using fem::Handle;

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

template <class F>
void parallel_for(int64_t n, F&& fn) {
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)std::max(1u, std::min(hw == 0 ? 1u : hw, 32u));
    if (n < 4096 || nt == 1) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi) break;
        pool.emplace_back([&fn, lo, hi] { fn(lo, hi); });
    }
    for (auto& th : pool) th.join();
}

struct Builder {
    Handle& h;
    int status = FEM_OK;
    explicit Builder(Handle& hh) : h(hh) {}

    template <class T>
    T* alloc(size_t n) {
        if (n == 0 || status != FEM_OK) return nullptr;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e != cudaSuccess) {
            fail(FEM_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
            return nullptr;
        }
        h.allocations.push_back(p);
        cudaMemset(p, 0, n * sizeof(T));
        return (T*)p;
    }
    template <class T>
    T* upload(const T* src, size_t n) {
        T* d = alloc<T>(n);
        if (d && src) {
            cudaError_t e = cudaMemcpy(d, src, n * sizeof(T), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) fail(FEM_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        }
        return d;
    }
    template <class T>
    T* upload(const std::vector<T>& v) {
        return upload(v.data(), v.size());
    }
    void fail(int code, const std::string& msg) {
        if (status == FEM_OK) {
            status = code;
            h.last_error = msg;
        }
    }
};

thread_local std::string g_error;

int set_error(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

}  // namespace

namespace fem {
int report(int code, const char* message) {
    g_error = message;
    return code;
}
int report_cuda(cudaError_t err) {
    if (err == cudaSuccess) return FEM_OK;
    g_error = std::string("CUDA error: ") + cudaGetErrorString(err);
    return FEM_ERR_CUDA;
}
}  // namespace fem

namespace {

int cuda_status(cudaError_t e, Handle* h = nullptr) {
    if (e == cudaSuccess) return FEM_OK;
    std::string msg = std::string("CUDA error: ") + cudaGetErrorString(e);
    if (h) h->last_error = msg;
    return set_error(FEM_ERR_CUDA, msg);
}


template <class T>
T* upload_plain(const std::vector<T>& v, std::vector<void*>& owned, cudaError_t& err) {
    if (v.empty() || err != cudaSuccess) return nullptr;
    void* p = nullptr;
    err = cudaMalloc(&p, v.size() * sizeof(T));
    if (err != cudaSuccess) return nullptr;
    owned.push_back(p);
    err = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return (T*)p;
}

// Re-register the surface contacts of a handle being replaced on the new one
// (topology rebuilds), refitted at q.
int carry_surfaces(const Handle& from, Handle& to, const float* q) {
    std::string why;
    const int nb = (int)from.sf_host_start.size();
    int code = fem::surface_register(to, nb, from.sf_host_start.data(), from.sf_host_size.data(),
                                     from.sf_host_toff.data(), from.sf_host_tris.data(), from.sf_ke, from.sf_kd, q,
                                     nullptr, why);
    if (code == FEM_ERR_BAD_ARG) return set_error(code, why);
    if (code == FEM_OK) {
        to.sf_host_start = from.sf_host_start;
        to.sf_host_size = from.sf_host_size;
        to.sf_host_toff = from.sf_host_toff;
        to.sf_host_tris = from.sf_host_tris;
        to.tangent_refreshes = from.tangent_refreshes;
    }
    return code;
}

// Register (or clear, capacity 0) the caller's soft-contact list; grows the
// per-contact scratch and allocates the per-node list heads on first use.
int register_soft_contacts(Handle& h, const int32_t* count, const int32_t* particle, const float* body_pos,
                           const float* body_vel, const float* normal, int32_t capacity) {
    if (capacity < 0) return set_error(FEM_ERR_BAD_ARG, "soft contact capacity must be non-negative");
    if (capacity > 0 && (!count || !particle || !body_pos || !body_vel || !normal))
        return set_error(FEM_ERR_BAD_ARG, "soft contact arrays are required for a non-zero capacity");
    if (capacity > 0 && h.P > 0) {
        auto grab = [&](size_t bytes, void** out) {
            cudaError_t e = cudaMalloc(out, bytes);
            if (e == cudaSuccess) h.allocations.push_back(*out);
            return e;
        };
        cudaError_t e = cudaSuccess;
        if (h.sc_head == nullptr) e = grab(sizeof(int) * (size_t)h.P, (void**)&h.sc_head);
        if (e == cudaSuccess && capacity > h.sc_alloc) {
            e = grab(sizeof(int) * (size_t)capacity, (void**)&h.sc_next);
            if (e == cudaSuccess) e = grab(sizeof(float4) * (size_t)capacity, (void**)&h.sc_force);
            if (e == cudaSuccess) h.sc_alloc = capacity;
        }
        if (e != cudaSuccess) return cuda_status(e, &h);
    }
    h.sc_count = count;
    h.sc_particle = particle;
    h.sc_pos = body_pos;
    h.sc_vel = body_vel;
    h.sc_normal = normal;
    h.sc_cap = capacity > 0 ? capacity : 0;
    return FEM_OK;
}

// Up to this many scenes keep each CTA's slices a contiguous run; more scenes
// (a batch) are dealt to the CTAs in up to kSceneChunks runs per scene.
constexpr int kContiguousScenes = 4;
constexpr int kSceneChunks = 16;

// Contiguous split of the slices over the CTAs that minimises the largest
// cost / speed, with at most Lmax slices per CTA: bisection on the makespan,
// each CTA taking (in order) every slice that still fits.
std::vector<int> split_slices(const std::vector<int64_t>& cost, const std::vector<double>& speed, int Lmax) {
    const int n = (int)cost.size(), G = (int)speed.size();
    std::vector<int> start(G + 1, n);
    auto place = [&](double T, std::vector<int>* out) {
        int sl = 0;
        for (int c = 0; c < G; ++c) {
            if (out) (*out)[c] = sl;
            const double budget = T * speed[c];
            double acc = 0.0;
            int taken = 0;
            while (sl < n && taken < Lmax && acc + (double)cost[sl] <= budget) {
                acc += (double)cost[sl];
                ++sl;
                ++taken;
            }
        }
        if (out) (*out)[G] = n;
        return sl == n;
    };
    double total = 0.0, vmin = 1e300;
    for (int64_t c : cost) total += (double)c;
    for (double v : speed) vmin = std::min(vmin, v);
    double lo = 0.0, hi = (total + 1.0) / std::max(vmin, 1e-30);
    if (!place(hi, nullptr)) {  // the slice cap binds: fall back to even counts
        for (int c = 0; c <= G; ++c) start[c] = (int)((int64_t)n * c / G);
        return start;
    }
    for (int it = 0; it < 64; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (place(mid, nullptr)) hi = mid;
        else lo = mid;
    }
    place(hi, &start);
    return start;
}

// (Re)compute the PCG grid for the handle's kernel variant, the per-(CTA,
// scene) segment tables of the deterministic reductions and the L2-resident
// slice count.  Allocates (at construction and on a tuning change only).
int configure_launch(Handle& h) {
    if (h.P == 0) return FEM_OK;
    for (void* p : h.launch_allocations) cudaFree(p);
    h.launch_allocations.clear();
    // L2-resident prefix of the matrix stream (40 bytes per stored block):
    // automatic (-2) keeps the whole matrix when it fits in 60% of L2 and none
    // otherwise, since pinning part of a larger matrix only evicts the vectors
    int64_t budget = h.l2_resident_bytes;
    if (budget < 0) {
        int dev = 0, l2 = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
        budget = (int64_t)(0.6 * (double)l2);
        if (h.l2_resident_bytes == -2) {
            const int64_t total = (int64_t)h.host_slice_ptr[h.nslices] * fem::kSlice * 40;
            budget = total <= budget ? total : 0;
        }
    }
    int64_t acc = 0;
    int rs = 0;
    for (int sl = 0; sl < h.nslices; ++sl) {
        int64_t bytes = (int64_t)(h.host_slice_ptr[sl + 1] - h.host_slice_ptr[sl]) * fem::kSlice * 40;
        if (acc + bytes > budget) break;
        acc += bytes;
        ++rs;
    }
    h.resident_slices = rs;
    cudaError_t err = fem::pcg_configure(h);
    if (err != cudaSuccess) return cuda_status(err, &h);
    h.rec0 = h.rec1 = h.p4 = h.s4 = h.w4 = nullptr;
    if (h.cg_variant == 1) {  // records and non-resident own-row state of the single-reduction variant
        std::vector<float4> zeros3(3 * (size_t)h.P, make_float4(0.f, 0.f, 0.f, 0.f));
        std::vector<float4> zeros1((size_t)h.P, make_float4(0.f, 0.f, 0.f, 0.f));
        h.rec0 = upload_plain(zeros3, h.launch_allocations, err);
        h.rec1 = upload_plain(zeros3, h.launch_allocations, err);
        if (!h.resident) {
            h.p4 = upload_plain(zeros1, h.launch_allocations, err);
            h.s4 = upload_plain(zeros1, h.launch_allocations, err);
            h.w4 = upload_plain(zeros1, h.launch_allocations, err);
        }
        if (err != cudaSuccess) return cuda_status(err, &h);
    }
    const std::vector<int>& slice_scene = h.host_slice_scene;
    const int nscenes = h.nscenes;
    // Slices per CTA, at most slices_per_cta each, balanced by slice cost (or by
    // calibrated speed, FEM_TUNE_BALANCE).  One scene, or a few: contiguous runs.
    // Many scenes (a batch): each scene is cut into up to kSceneChunks runs, the
    // runs are interleaved (run 0 of every scene, then run 1, ...) and that
    // sequence is split into contiguous pieces; so once most scenes have
    // converged, the rows still iterating are spread over many CTAs instead of
    // the two or three that would own a scene's contiguous slices.
    {
        std::vector<double> speed(h.grid, 1.0);
        if (h.balance && (int)h.cta_speed.size() == h.grid) speed = h.cta_speed;
        std::vector<int> order(h.nslices);
        for (int sl = 0; sl < h.nslices; ++sl) order[sl] = sl;
        h.cta_contiguous = nscenes <= kContiguousScenes ? 1 : 0;
        if (!h.cta_contiguous) {
            std::vector<int> s0(nscenes + 1, 0);
            for (int sl = 0; sl < h.nslices; ++sl) s0[slice_scene[sl] + 1]++;
            for (int sc = 0; sc < nscenes; ++sc) s0[sc + 1] += s0[sc];
            order.clear();
            for (int j = 0; j < kSceneChunks; ++j)
                for (int sc = 0; sc < nscenes; ++sc) {
                    const int n = s0[sc + 1] - s0[sc], k = std::min(kSceneChunks, n);
                    if (j >= k) continue;
                    for (int sl = s0[sc] + (int)((int64_t)n * j / k); sl < s0[sc] + (int)((int64_t)n * (j + 1) / k); ++sl)
                        order.push_back(sl);
                }
        }
        std::vector<int64_t> cost(h.nslices);
        for (int i = 0; i < h.nslices; ++i) cost[i] = h.host_slice_cost[order[i]];
        h.host_cta_slice0 = split_slices(cost, speed, h.slices_per_cta);
        int widest = 0;
        for (int c = 0; c < h.grid; ++c) {
            widest = std::max(widest, h.host_cta_slice0[c + 1] - h.host_cta_slice0[c]);
            std::sort(order.begin() + h.host_cta_slice0[c], order.begin() + h.host_cta_slice0[c + 1]);
        }
        if (widest > h.slices_per_cta) return set_error(FEM_ERR_CUDA, "slice split exceeds the per-CTA capacity");
        h.host_cta_list = order;
        h.cta_slice0 = upload_plain(h.host_cta_slice0, h.launch_allocations, err);
        h.cta_list = upload_plain(h.host_cta_list, h.launch_allocations, err);
    }
    // Segments: the runs of one scene in a CTA's (ascending) slice list.  Their
    // partials go to the segment buffer scene-major, ordered by CTA within a
    // scene, so every per-scene total sums the same values in the same order.
    std::vector<int> cta_seg_base(h.grid + 1, 0), seg_start, seg_scene, scene_seg0(nscenes + 1, 0);
    for (int c = 0; c < h.grid; ++c) {
        cta_seg_base[c] = (int)seg_start.size();
        for (int i = h.host_cta_slice0[c]; i < h.host_cta_slice0[c + 1]; ++i) {
            const int sc = slice_scene[h.host_cta_list[i]];
            if (i == h.host_cta_slice0[c] || sc != seg_scene.back()) {
                seg_start.push_back(i);
                seg_scene.push_back(sc);
                scene_seg0[sc + 1]++;
            }
        }
    }
    const int nseg = (int)seg_start.size();
    cta_seg_base[h.grid] = nseg;
    for (int sc = 0; sc < nscenes; ++sc) scene_seg0[sc + 1] += scene_seg0[sc];
    std::vector<int> seg_pos(nseg), fill(scene_seg0.begin(), scene_seg0.end() - 1);
    for (int t = 0; t < nseg; ++t) seg_pos[t] = fill[seg_scene[t]]++;
    h.nseg = nseg;
    h.cta_seg_base = upload_plain(cta_seg_base, h.launch_allocations, err);
    h.seg_start = upload_plain(seg_start, h.launch_allocations, err);
    h.seg_pos = upload_plain(seg_pos, h.launch_allocations, err);
    h.scene_seg0 = upload_plain(scene_seg0, h.launch_allocations, err);
    std::vector<float> zeros(2 * 3 * (size_t)std::max(1, nseg), 0.0f);
    h.seg_part = upload_plain(zeros, h.launch_allocations, err);
    if (err != cudaSuccess) return cuda_status(err, &h);
    return FEM_OK;
}

// Measure each CTA's SpMV-phase speed on 10-iteration solves of a synthetic
// right-hand side and re-split the slices by it; a few rounds, keeping the
// split with the smallest slowest-CTA time.  Host-synchronous; runs on the
// legacy stream.
int calibrate_balance(Handle& h) {
    if (h.P == 0 || h.grid < 2) return FEM_OK;
    const int rounds = 4;
    std::vector<float> ones(3 * (size_t)h.P, 1.0f);
    float *rhs = nullptr, *x = nullptr;
    unsigned long long* times = nullptr;
    cudaError_t e = cudaMalloc(&rhs, sizeof(float) * ones.size());
    if (e == cudaSuccess) e = cudaMalloc(&x, sizeof(float) * ones.size());
    if (e == cudaSuccess) e = cudaMalloc(&times, sizeof(unsigned long long) * 2 * (size_t)h.grid);
    if (e == cudaSuccess) e = cudaMemcpy(rhs, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice);
    std::vector<double> speed(h.grid, 1.0), best_speed = speed;
    double best = 1e300;
    int code = FEM_OK;
    for (int round = 0; round < rounds && e == cudaSuccess && code == FEM_OK; ++round) {
        h.cta_speed = speed;
        code = configure_launch(h);
        if (code != FEM_OK) break;
        e = cudaMemset(times, 0, sizeof(unsigned long long) * 2 * (size_t)h.grid);
        if (e != cudaSuccess) break;
        h.cta_time = times;
        e = fem::launch_pcg(h, h.dt, 0, nullptr, nullptr, nullptr, nullptr, rhs, x, 1e-30f, 10, false);
        h.cta_time = nullptr;
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        std::vector<unsigned long long> t(2 * (size_t)h.grid);
        if (e == cudaSuccess)
            e = cudaMemcpy(t.data(), times, sizeof(unsigned long long) * t.size(), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) break;
        double worst = 0.0;
        std::vector<double> next = speed;
        for (int c = 0; c < h.grid; ++c) {
            int64_t cost = 0;
            for (int i = h.host_cta_slice0[c]; i < h.host_cta_slice0[c + 1]; ++i)
                cost += h.host_slice_cost[h.host_cta_list[i]];
            if (cost == 0 || t[2 * c + 1] == 0) continue;
            const double per_iter = (double)t[2 * c] / (double)t[2 * c + 1];
            worst = std::max(worst, per_iter);
            if (per_iter > 0.0) next[c] = (double)cost / per_iter;
        }
        if (worst < best) {
            best = worst;
            best_speed = speed;
        }
        speed = next;
    }
    cudaFree(rhs);
    cudaFree(x);
    cudaFree(times);
    if (e != cudaSuccess) return cuda_status(e, &h);
    if (code != FEM_OK) return code;
    h.cta_speed = best_speed;
    return configure_launch(h);
}

}  // namespace

extern "C" {

const char* fem_version(void) { return "fem_gb300 0.1 (sm_103a)"; }

const char* fem_status_string(int status) {
    switch (status) {
        case FEM_OK: return "ok";
        case FEM_ERR_BAD_ARG: return g_error.empty() ? "bad argument" : g_error.c_str();
        case FEM_ERR_NOT_CONVERGED: return "linear solve reached maxiter above tolerance";
        case FEM_ERR_NON_FINITE: return "non-finite value in the linear solve";
        case FEM_ERR_TIMEOUT: return "a bounded device wait timed out";
        case FEM_ERR_CUDA: return g_error.empty() ? "CUDA error" : g_error.c_str();
        case FEM_ERR_UNSUPPORTED: return g_error.empty() ? "unsupported option" : g_error.c_str();
        default: return "unknown status";
    }
}

}  // extern "C"

// Construction.  `candidate` (streaming Tet4 assembly) gives, per row, the sorted
// columns the pattern reserves; every triplet's column must be among them, and
// reserved entries without contributors hold exact zeros.
int fem::create_handle(const FemDesc* d, const std::vector<std::vector<int>>* candidate, FemHandle** out) {
    if (d == nullptr || out == nullptr) return set_error(FEM_ERR_BAD_ARG, "null descriptor or output");
    *out = nullptr;
    const int P = d->particle_count, T = d->tet_count, Hn = d->hex_count, S = d->spring_count, Tri = d->tri_count;
    if (P < 0 || T < 0 || Hn < 0 || S < 0 || Tri < 0) return set_error(FEM_ERR_BAD_ARG, "negative element count");
    if (P > 0 && (d->particle_q == nullptr || d->particle_mass == nullptr || d->particle_inv_mass == nullptr))
        return set_error(FEM_ERR_BAD_ARG, "particle arrays are required");
    if (T > 0 && (d->tet_indices == nullptr || d->tet_poses == nullptr || d->tet_materials == nullptr))
        return set_error(FEM_ERR_BAD_ARG, "tet arrays are required");
    if (Hn > 0 && (d->hex_indices == nullptr || d->hex_materials == nullptr || d->hex_inv_J0 == nullptr ||
                   d->hex_det_J0_w == nullptr))
        return set_error(FEM_ERR_BAD_ARG, "hex arrays are required");
    if (S > 0 && (d->spring_indices == nullptr || d->spring_rest_length == nullptr ||
                  d->spring_stiffness == nullptr || d->spring_damping == nullptr))
        return set_error(FEM_ERR_BAD_ARG, "spring arrays are required");
    if (Tri > 0 && (d->tri_indices == nullptr || d->tri_poses == nullptr || d->tri_materials == nullptr))
        return set_error(FEM_ERR_BAD_ARG, "triangle arrays are required");
    const bool torque = S > 0 && d->spring_rest_direction != nullptr && d->torque_stiffness > 0.0f;
    if (d->particle_contact && !(2.0f * d->particle_max_radius + d->particle_cohesion > 0.0f))
        return set_error(FEM_ERR_BAD_ARG, "particle contact needs 2 max_radius + cohesion > 0");
    if (!(d->tolerance > 0.0f) || !std::isfinite(d->tolerance))
        return set_error(FEM_ERR_BAD_ARG, "linear_solver_tolerance must be finite and positive");
    if (d->maxiter < 0) return set_error(FEM_ERR_BAD_ARG, "linear_solver_maxiter must be non-negative");
    if (d->preconditioner != FEM_PRECOND_BLOCK_DIAG && d->preconditioner != FEM_PRECOND_DIAG)
        return set_error(FEM_ERR_UNSUPPORTED, "preconditioner must be block_diag or diag");
    const int64_t ntrip = (int64_t)P + 2 * (int64_t)S + 3 * (int64_t)Tri + 16 * (int64_t)T + 64 * (int64_t)Hn;
    if (4 * (int64_t)T + 8 * (int64_t)Hn + 3 * (int64_t)Tri >= (int64_t)INT32_MAX)
        return set_error(FEM_ERR_BAD_ARG, "problem too large for int32 element slots");
    if (ntrip >= (int64_t)INT32_MAX) return set_error(FEM_ERR_BAD_ARG, "problem too large for int32 triplet ids");
    for (int64_t k = 0; k < 4 * (int64_t)T; ++k)
        if (d->tet_indices[k] < 0 || d->tet_indices[k] >= P) return set_error(FEM_ERR_BAD_ARG, "tet index out of range");
    for (int64_t k = 0; k < 8 * (int64_t)Hn; ++k)
        if (d->hex_indices[k] < 0 || d->hex_indices[k] >= P) return set_error(FEM_ERR_BAD_ARG, "hex index out of range");
    for (int64_t k = 0; k < 2 * (int64_t)S; ++k)
        if (d->spring_indices[k] >= P || d->spring_indices[k] < -1)
            return set_error(FEM_ERR_BAD_ARG, "spring index out of range");
    for (int64_t k = 0; k < 3 * (int64_t)Tri; ++k)
        if (d->tri_indices[k] < 0 || d->tri_indices[k] >= P)
            return set_error(FEM_ERR_BAD_ARG, "triangle index out of range");
    std::vector<unsigned char> fixed_mask(P, 0);
    for (int k = 0; k < d->fixed_count; ++k) {
        int i = d->fixed_indices[k];
        if (i < 0 || i >= P) return set_error(FEM_ERR_BAD_ARG, "fixed_particle_indices contains an out-of-range node");
        fixed_mask[i] = 1;
    }
    std::vector<int64_t> scenes;
    if (d->scene_offsets != nullptr && d->scene_count > 0) {
        scenes.assign(d->scene_offsets, d->scene_offsets + d->scene_count + 1);
        if (scenes.front() != 0 || scenes.back() != P) return set_error(FEM_ERR_BAD_ARG, "scene offsets must span [0, P]");
        for (int s = 0; s < d->scene_count; ++s)
            if (scenes[s + 1] <= scenes[s]) return set_error(FEM_ERR_BAD_ARG, "scene offsets must increase");
    } else {
        scenes = {0, (int64_t)P};
    }
    const int nscenes = (int)scenes.size() - 1;
    if (nscenes > 1024) return set_error(FEM_ERR_UNSUPPORTED, "at most 1024 scenes per handle");
    if (P > 0) {
        // elements and springs may not couple scenes
        std::vector<int> scene_of(P);
        for (int s = 0; s < nscenes; ++s)
            for (int64_t i = scenes[s]; i < scenes[s + 1]; ++i) scene_of[i] = s;
        auto same = [&](const int32_t* idx, int width, int64_t count) {
            for (int64_t e = 0; e < count; ++e) {
                int s0 = -1;
                for (int k = 0; k < width; ++k) {
                    int n = idx[e * width + k];
                    if (n < 0) continue;
                    if (s0 < 0) s0 = scene_of[n];
                    else if (scene_of[n] != s0) return false;
                }
            }
            return true;
        };
        if (!same(d->tet_indices, 4, T) || !same(d->hex_indices, 8, Hn) || !same(d->spring_indices, 2, S) ||
            !same(d->tri_indices, 3, Tri))
            return set_error(FEM_ERR_BAD_ARG, "an element or spring couples two scenes");
        if (d->particle_contact && nscenes > 1)
            return set_error(FEM_ERR_UNSUPPORTED, "particle contact couples scenes; use one scene");
    }

    int device = 0;
    cudaError_t ce = cudaGetDevice(&device);
    if (ce != cudaSuccess) return cuda_status(ce);
    auto* H = new FemHandle();
    H->device = device;
    Handle& h = H->h;
    Builder b(h);
    h.P = P;
    h.T = T;
    h.H = Hn;
    h.S = S;
    h.Tri = Tri;
    h.nscenes = nscenes;
    h.ntrip = ntrip;
    h.dt = d->dt;
    h.min_stretch = d->min_stretch;
    h.max_stretch = d->max_stretch;
    h.has_ground = d->has_ground;
    for (int k = 0; k < 4; ++k) h.ground[k] = d->ground_plane[k];
    h.gke = d->ground_ke;
    h.gkd = d->ground_kd;
    h.gkf = d->ground_kf;
    h.gmu = d->ground_mu;
    h.linear_damping = d->linear_damping;
    h.enable_act = d->enable_tet_activations;
    h.precond = d->preconditioner;
    h.maxiter = d->maxiter;
    h.tol = d->tolerance;
    h.nfixed = d->fixed_count;
    h.torque_ke = d->torque_stiffness;
    h.torque_kd = d->torque_damping;
    h.pcontact = d->particle_contact != 0 && P > 1;
    h.pke = d->particle_ke;
    h.pkd = d->particle_kd;
    h.pkf = d->particle_kf;
    h.pmu = d->particle_mu;
    h.pcoh = d->particle_cohesion;
    h.pmaxr = d->particle_max_radius;
    h.ske = d->soft_contact_ke;
    h.skd = d->soft_contact_kd;
    h.skf = d->soft_contact_kf;
    h.smu = d->soft_contact_mu;
    fem::upload_hex_reference_table();
    fem::upload_hex_reference_table_adjoint();

    // ---- empty-material tets produce no triplets (kernels.py:690-700)
    std::vector<unsigned char> tet_empty(T, 0);
    for (int t = 0; t < T; ++t)
        tet_empty[t] = d->tet_materials[3 * t] == 0.0f && d->tet_materials[3 * t + 1] == 0.0f &&
                       d->tet_materials[3 * t + 2] == 0.0f;
    // triplet regions [P | 2S | 3Tri | 16T | 64H] (solver.py:312-321, 1015-1136)
    const int64_t off_spring = P, off_tri = (int64_t)P + 2 * (int64_t)S, off_tet = off_tri + 3 * (int64_t)Tri,
                  off_hex = off_tet + 16 * (int64_t)T;
    auto trip_rc = [&](int64_t t, int& r, int& c) {
        if (t < off_spring) {
            r = c = (int)t;
        } else if (t < off_tri) {
            int64_t k = t - off_spring;
            int s = (int)(k >> 1);
            int a = d->spring_indices[2 * s], bb = d->spring_indices[2 * s + 1];
            if (k & 1) { r = bb; c = a; } else { r = a; c = bb; }
            if (r < 0 || c < 0) r = c = -1;
        } else if (t < off_tet) {
            r = c = d->tri_indices[t - off_tri];
        } else if (t < off_hex) {
            int64_t k = t - off_tet;
            int e = (int)(k >> 4), ab = (int)(k & 15);
            if (tet_empty[e]) { r = c = -1; return; }
            r = d->tet_indices[4 * e + (ab >> 2)];
            c = d->tet_indices[4 * e + (ab & 3)];
        } else {
            int64_t k = t - off_hex;
            int e = (int)(k >> 6), ab = (int)(k & 63);
            r = d->hex_indices[8 * e + (ab >> 3)];
            c = d->hex_indices[8 * e + (ab & 7)];
        }
    };

    // ---- pattern: bucket triplets by row (ascending id), sort each row by column
    std::vector<int> trip_rows(ntrip), trip_cols(ntrip);
    std::vector<int64_t> row_ptr(P + 1, 0);
    for (int64_t t = 0; t < ntrip; ++t) {
        int r, c;
        trip_rc(t, r, c);
        trip_rows[t] = r;
        trip_cols[t] = c;
        if (r >= 0) row_ptr[r + 1]++;
    }
    for (int i = 0; i < P; ++i) row_ptr[i + 1] += row_ptr[i];
    const int64_t nvalid = P > 0 ? row_ptr[P] : 0;
    std::vector<int> contrib(nvalid);
    {
        std::vector<int64_t> pos(row_ptr.begin(), row_ptr.end() - 1);
        for (int64_t t = 0; t < ntrip; ++t)
            if (trip_rows[t] >= 0) contrib[pos[trip_rows[t]]++] = (int)t;
    }
    std::vector<int> row_nnz(P, 0);
    std::vector<unsigned char> outside(P, 0);
    parallel_for(P, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            int* beg = contrib.data() + row_ptr[i];
            int* end = contrib.data() + row_ptr[i + 1];
            std::stable_sort(beg, end, [&](int x, int y) { return trip_cols[x] < trip_cols[y]; });
            if (candidate != nullptr) {
                const std::vector<int>& cc = (*candidate)[i];
                size_t k = 0;
                for (int* p = beg; p != end; ++p) {
                    while (k < cc.size() && cc[k] < trip_cols[*p]) ++k;
                    if (k == cc.size() || cc[k] != trip_cols[*p]) outside[i] = 1;
                }
                row_nnz[i] = (int)cc.size();
                continue;
            }
            int n = 0, prev = -1;
            for (int* p = beg; p != end; ++p)
                if (trip_cols[*p] != prev) { ++n; prev = trip_cols[*p]; }
            row_nnz[i] = n;
        }
    });
    if (std::find(outside.begin(), outside.end(), 1) != outside.end()) {
        fem_destroy(H);
        return set_error(FEM_ERR_BAD_ARG, "a block lies outside the reserved sparse pattern");
    }
    std::vector<int> bsr_offsets(P + 1, 0);
    for (int i = 0; i < P; ++i) bsr_offsets[i + 1] = bsr_offsets[i] + row_nnz[i];
    const int64_t nnzb = bsr_offsets[P];
    h.nnzb = nnzb;
    std::vector<int> bsr_columns(nnzb), slot_cptr(nnzb + 1);
    slot_cptr[nnzb] = (int)nvalid;
    parallel_for(P, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            if (candidate != nullptr) {
                const std::vector<int>& cc = (*candidate)[i];
                int64_t p = row_ptr[i];
                for (size_t k = 0; k < cc.size(); ++k) {
                    const int slot = bsr_offsets[i] + (int)k;
                    bsr_columns[slot] = cc[k];
                    slot_cptr[slot] = (int)p;
                    while (p < row_ptr[i + 1] && trip_cols[contrib[p]] == cc[k]) ++p;
                }
                continue;
            }
            int slot = bsr_offsets[i] - 1, prev = -1;
            for (int64_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
                int c = trip_cols[contrib[p]];
                if (c != prev) {
                    ++slot;
                    bsr_columns[slot] = c;
                    slot_cptr[slot] = (int)p;
                    prev = c;
                }
            }
        }
    });

    // ---- SELL-32 layout, sliced per scene
    std::vector<int> slice_ptr(1, 0), slice_scene;
    std::vector<int2> slice_meta;
    for (int s = 0; s < nscenes; ++s) {
        for (int64_t r0 = scenes[s]; r0 < scenes[s + 1]; r0 += fem::kSlice) {
            int n = (int)std::min<int64_t>(fem::kSlice, scenes[s + 1] - r0);
            int w = 0;
            for (int l = 0; l < n; ++l) w = std::max(w, row_nnz[r0 + l]);
            slice_meta.push_back(make_int2((int)r0, n));
            slice_scene.push_back(s);
            slice_ptr.push_back(slice_ptr.back() + w);
        }
    }
    h.nslices = (int)slice_meta.size();
    const int64_t nsell = (int64_t)slice_ptr.back() * fem::kSlice;
    h.nsell = nsell;
    std::vector<int> sell_slot(nsell, -1), sell_row(nsell, -1), scol(nsell, 0), slot_sell(nnzb);
    std::vector<unsigned> row_info(P);
    parallel_for(h.nslices, [&](int64_t lo, int64_t hi) {
        for (int64_t sl = lo; sl < hi; ++sl) {
            int w = slice_ptr[sl + 1] - slice_ptr[sl];
            for (int l = 0; l < fem::kSlice; ++l) {
                int r = slice_meta[sl].x + l;
                bool live = l < slice_meta[sl].y;
                for (int k = 0; k < w; ++k) {
                    int64_t e = ((int64_t)slice_ptr[sl] + k) * fem::kSlice + l;
                    if (!live) continue;
                    sell_row[e] = r;
                    scol[e] = r;
                    if (k < row_nnz[r]) {
                        int slot = bsr_offsets[r] + k;
                        sell_slot[e] = slot;
                        slot_sell[slot] = (int)e;
                        scol[e] = bsr_columns[slot];
                    }
                }
                if (live) row_info[r] = (unsigned)row_nnz[r] | (fixed_mask[r] ? fem::kFixedBit : 0u);
            }
        }
    });

    // ---- node incidence (element-force slots, springs), ascending order
    std::vector<int> elem_ptr(P + 1, 0), spring_ptr(P + 1, 0);
    for (int64_t k = 0; k < 4 * (int64_t)T; ++k) elem_ptr[d->tet_indices[k] + 1]++;
    for (int64_t k = 0; k < 8 * (int64_t)Hn; ++k) elem_ptr[d->hex_indices[k] + 1]++;
    for (int64_t k = 0; k < 3 * (int64_t)Tri; ++k) elem_ptr[d->tri_indices[k] + 1]++;
    for (int s = 0; s < S; ++s) {
        int a = d->spring_indices[2 * s], bb = d->spring_indices[2 * s + 1];
        if (a >= 0) spring_ptr[a + 1]++;
        if (bb >= 0 && bb != a) spring_ptr[bb + 1]++;
    }
    for (int i = 0; i < P; ++i) {
        elem_ptr[i + 1] += elem_ptr[i];
        spring_ptr[i + 1] += spring_ptr[i];
    }
    std::vector<int> elem_ent(elem_ptr[P]), spring_ent(spring_ptr[P]);
    {
        std::vector<int> pos(elem_ptr.begin(), elem_ptr.end() - 1);
        for (int64_t k = 0; k < 4 * (int64_t)T; ++k) elem_ent[pos[d->tet_indices[k]]++] = (int)k;
        for (int64_t k = 0; k < 8 * (int64_t)Hn; ++k) elem_ent[pos[d->hex_indices[k]]++] = (int)(4 * (int64_t)T + k);
        const int64_t tri0 = 4 * (int64_t)T + 8 * (int64_t)Hn;
        for (int64_t k = 0; k < 3 * (int64_t)Tri; ++k) elem_ent[pos[d->tri_indices[k]]++] = (int)(tri0 + k);
        std::vector<int> sp(spring_ptr.begin(), spring_ptr.end() - 1);
        for (int s = 0; s < S; ++s) {
            int a = d->spring_indices[2 * s], bb = d->spring_indices[2 * s + 1];
            if (a >= 0) spring_ent[sp[a]++] = 2 * s;
            if (bb >= 0 && bb != a) spring_ent[sp[bb]++] = 2 * s + 1;
        }
    }

    // ---- device data
    std::vector<float> radius(P, 0.0f);
    if (d->particle_radius) std::copy(d->particle_radius, d->particle_radius + P, radius.begin());
    std::vector<int> flags(P, 1);
    if (d->particle_flags) std::copy(d->particle_flags, d->particle_flags + P, flags.begin());
    h.rest = b.upload(d->particle_q, 3 * (size_t)P);
    h.mass = b.upload(d->particle_mass, P);
    h.inv_mass = b.upload(d->particle_inv_mass, P);
    h.radius = b.upload(radius);
    h.flags = b.upload(flags);
    h.fixed_mask = b.upload(fixed_mask);
    h.fixed_idx = b.upload(d->fixed_indices, (size_t)std::max(0, d->fixed_count));
    h.gravity_dev = b.alloc<float>(3);
    h.tet_idx = reinterpret_cast<int4*>(b.upload(d->tet_indices, 4 * (size_t)T));
    h.tet_pose = b.upload(d->tet_poses, 9 * (size_t)T);
    h.tet_mat = b.upload(d->tet_materials, 3 * (size_t)T);
    h.hex_idx = b.upload(d->hex_indices, 8 * (size_t)Hn);
    h.hex_invJ = b.upload(d->hex_inv_J0, 72 * (size_t)Hn);
    h.hex_detw = b.upload(d->hex_det_J0_w, 8 * (size_t)Hn);
    h.hex_mat = b.upload(d->hex_materials, 3 * (size_t)Hn);
    h.spring_idx = b.upload(d->spring_indices, 2 * (size_t)S);
    h.spring_rest = b.upload(d->spring_rest_length, S);
    h.spring_ke = b.upload(d->spring_stiffness, S);
    h.spring_kd = b.upload(d->spring_damping, S);
    if (torque) h.spring_dir = b.upload(d->spring_rest_direction, 3 * (size_t)S);
    h.tri_idx = b.upload(d->tri_indices, 3 * (size_t)Tri);
    h.tri_pose = reinterpret_cast<float4*>(b.upload(d->tri_poses, 4 * (size_t)Tri));
    h.tri_mat = b.upload(d->tri_materials, 5 * (size_t)Tri);
    if (h.pcontact) {
        h.grid_dim = fem::particle_grid_dim(P);
        const int64_t nb = (int64_t)h.grid_dim * h.grid_dim * h.grid_dim;
        h.grid_count = b.alloc<int>((size_t)nb);
        h.grid_start = b.alloc<int>((size_t)nb + 1);
        h.grid_part = b.alloc<int>((size_t)fem::scan_partial_count(nb));
        h.grid_items = b.alloc<int>(P);
        h.cell_of = b.alloc<int>(P);
        h.pforce = b.alloc<float4>(P);
    }
    h.node_elem_ptr = b.upload(elem_ptr);
    h.node_elem_ent = b.upload(elem_ent);
    h.node_spring_ptr = b.upload(spring_ptr);
    h.node_spring_ent = b.upload(spring_ent);
    h.elem_force = b.alloc<float4>(4 * (size_t)T + 8 * (size_t)Hn + 3 * (size_t)Tri);
    h.q4 = b.alloc<float4>(P);
    h.v4 = b.alloc<float4>(P);
    h.trip.a = b.alloc<float4>((size_t)ntrip);
    h.trip.b = b.alloc<float4>((size_t)ntrip);
    h.trip.c = b.alloc<float>((size_t)ntrip);
    h.trip_rows = b.upload(trip_rows);
    h.trip_cols = b.upload(trip_cols);
    // contributor lists keyed by SELL entry (empty for padding), so the
    // assembly reads entry -> range -> triplet ids with no slot indirection
    {
        std::vector<int> sell_cptr(nsell + 1, 0);
        parallel_for(nsell, [&](int64_t lo, int64_t hi) {
            for (int64_t e = lo; e < hi; ++e) {
                int slot = sell_slot[e];
                sell_cptr[e + 1] = slot < 0 ? 0 : slot_cptr[slot + 1] - slot_cptr[slot];
            }
        });
        for (int64_t e = 0; e < nsell; ++e) sell_cptr[e + 1] += sell_cptr[e];
        std::vector<int> sell_contrib(sell_cptr[nsell]);
        parallel_for(nsell, [&](int64_t lo, int64_t hi) {
            for (int64_t e = lo; e < hi; ++e) {
                int slot = sell_slot[e];
                if (slot >= 0)
                    std::copy(contrib.begin() + slot_cptr[slot], contrib.begin() + slot_cptr[slot + 1],
                              sell_contrib.begin() + sell_cptr[e]);
            }
        });
        h.sell_cptr = b.upload(sell_cptr);
        h.sell_contrib = b.upload(sell_contrib);
    }
    h.sell_slot = b.upload(sell_slot);
    h.sell_row = b.upload(sell_row);
    h.bsr_offsets = b.upload(bsr_offsets);
    h.bsr_columns = b.upload(bsr_columns);
    h.slot_sell = b.upload(slot_sell);
    h.valA = b.alloc<float4>(nsell);
    h.valB = b.alloc<float4>(nsell);
    h.valC = b.alloc<float>(nsell);
    h.scol = b.upload(scol);
    {  // 16-bit column offsets for the PCG when every stored block's offset fits
        bool fits = true;
        std::vector<short> dcol(nsell, 0);
        for (int64_t e = 0; e < nsell && fits; ++e) {
            if (sell_row[e] < 0) continue;
            const int d = scol[e] - sell_row[e];
            if (d < -32768 || d > 32767) fits = false;
            else dcol[e] = (short)d;
        }
        if (fits && nsell > 0) {
            h.dcol = b.upload(dcol);
            // slots k < 64 at which every live row of a slice has the same offset
            std::vector<unsigned long long> kmask(h.nslices, 0ull);
            std::vector<short> kval((size_t)h.nslices * 64, 0);
            for (int sl = 0; sl < h.nslices; ++sl) {
                const int w = std::min(64, slice_ptr[sl + 1] - slice_ptr[sl]);
                for (int k = 0; k < w; ++k) {
                    bool any = false, same = true;
                    short v = 0;
                    int rows = 0;
                    for (int l = 0; l < slice_meta[sl].y && same; ++l) {
                        if (k >= row_nnz[slice_meta[sl].x + l]) continue;
                        const short d = dcol[((int64_t)slice_ptr[sl] + k) * fem::kSlice + l];
                        if (!any) v = d;
                        same = !any || d == v;
                        any = true;
                        ++rows;
                    }
                    if (any && same) {
                        kmask[sl] |= 1ull << k;
                        kval[(size_t)sl * 64 + k] = v;
                        h.uniform_blocks += rows;
                    }
                }
            }
            h.slice_kmask = b.upload(kmask);
            h.slice_kval = b.upload(kval);
        }
    }
    {  // per (slice, k): the lanes whose column at k is a fixed node (fem_apply_operator's mask)
        std::vector<unsigned> fixcol(nsell / fem::kSlice, 0u);
        bool any = false;
        for (int sl = 0; sl < h.nslices; ++sl)
            for (int k = 0; k < slice_ptr[sl + 1] - slice_ptr[sl]; ++k)
                for (int l = 0; l < slice_meta[sl].y; ++l) {
                    const int r = slice_meta[sl].x + l;
                    if (k >= row_nnz[r]) continue;
                    if (fixed_mask[scol[((int64_t)slice_ptr[sl] + k) * fem::kSlice + l]]) {
                        fixcol[(size_t)slice_ptr[sl] + k] |= 1u << l;
                        any = true;
                    }
                }
        if (any) h.fixcol = b.upload(fixcol);
    }
    h.slice_ptr = b.upload(slice_ptr);
    h.slice_meta = b.upload(slice_meta);
    h.slice_scene = b.upload(slice_scene);
    h.row_info = b.upload(row_info);
    h.minv = b.alloc<float>(9 * (size_t)P);
    h.x = b.alloc<float4>(P);
    h.r = b.alloc<float4>(P);
    h.zp0 = b.alloc<float4>(2 * (size_t)P);
    h.zp1 = b.alloc<float4>(2 * (size_t)P);
    h.stage = b.alloc<float4>(2 * (size_t)P);
    if (d->velocity_increment != nullptr) {
        h.dv = d->velocity_increment;
        h.dv_owned = false;
        if (P > 0) cudaMemset(h.dv, 0, sizeof(float) * 3 * (size_t)P);
    } else {
        h.dv = b.alloc<float>(3 * (size_t)P);
    }
    h.barrier = b.alloc<unsigned>(1);
    h.status = b.alloc<int>(1);
    h.scene_stats = b.alloc<fem::SceneStats>(nscenes);
    h.cum_iters = b.alloc<long long>(nscenes);
    h.resid_max = b.alloc<float>(2);
    if (b.status != FEM_OK) {
        int code = b.status;
        g_error = h.last_error;
        fem_destroy(H);
        return code;
    }
    if (P > 0) {
        cudaError_t ge = cudaMemcpy(h.gravity_dev, d->gravity, sizeof(float) * 3, cudaMemcpyHostToDevice);
        if (ge != cudaSuccess) {
            fem_destroy(H);
            return cuda_status(ge);
        }
    }

    // ---- launch configuration and deterministic-reduction segment tables
    h.host_slice_scene = slice_scene;
    h.host_slice_ptr = slice_ptr;
    h.host_slice_cost.assign(h.nslices, 0);
    for (int sl = 0; sl < h.nslices; ++sl)
        for (int l = 0; l < slice_meta[sl].y; ++l) h.host_slice_cost[sl] += row_nnz[slice_meta[sl].x + l] + 4;
    int code = configure_launch(h);
    if (code != FEM_OK) {
        g_error = h.last_error;
        fem_destroy(H);
        return code;
    }
    cudaError_t err = cudaSuccess;

    // ---- initial assembly at the construction positions (solver.py:330-341)
    cudaStream_t s0 = nullptr;
    err = fem::launch_node_prepare(h, h.rest, nullptr, false, false, false, s0);
    if (err == cudaSuccess) err = fem::launch_constant_blocks(h, h.dt, s0);
    if (err == cudaSuccess) err = fem::launch_element_tangent(h, h.dt, s0);
    if (err == cudaSuccess) err = fem::launch_gather(h, s0);
    if (err == cudaSuccess) err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        int code = cuda_status(err);
        fem_destroy(H);
        return code;
    }
    *out = H;
    return FEM_OK;
}

extern "C" {

int fem_create(const FemDesc* d, FemHandle** out) { return fem::create_handle(d, nullptr, out); }

int fem_destroy(FemHandle* H) {
    if (H == nullptr) return FEM_OK;
    DeviceGuard g(H->device);
    for (cudaEvent_t e : H->h.timing_events) cudaEventDestroy(e);
    for (void* p : H->h.launch_allocations) cudaFree(p);
    for (void* p : H->h.allocations) cudaFree(p);
    delete H;
    return FEM_OK;
}

int fem_step(FemHandle* H, float* q_in, float* v_in, float* q_out, float* v_out, float* f_ws,
             const float* external_forces, const float* activations, const float* gravity, float dt, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    if (!q_in || !v_in || !q_out || !v_out || !f_ws) return set_error(FEM_ERR_BAD_ARG, "null state pointer");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return set_error(FEM_ERR_BAD_ARG, "dt must be finite and positive");
    if (h.enable_act && h.T > 0 && activations == nullptr)
        return set_error(FEM_ERR_BAD_ARG, "tet activations are enabled but none were passed");
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = fem::launch_node_prepare(h, q_in, v_in, true, true, true, s);
    if (err == cudaSuccess) err = fem::launch_element_forces(h, activations, s);
    if (err == cudaSuccess)
        err = fem::launch_node_forces(h, external_forces, gravity, dt, FEM_TERM_ALL, true, f_ws, s);
    bool timed = false;
    if (err == cudaSuccess && h.timing) {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(s, &cap);
        if (cap == cudaStreamCaptureStatusNone) {
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            h.timing_events.push_back(e0);
            h.timing_events.push_back(e1);
            cudaEventRecord(e0, s);
            timed = true;
        }
    }
    if (err == cudaSuccess) err = fem::launch_pcg(h, dt, 1, q_out, v_out, f_ws, s);
    if (timed) cudaEventRecord(h.timing_events.back(), s);
    return cuda_status(err, &h);
}

int fem_set_soft_contacts(FemHandle* H, const int32_t* count, const int32_t* particle, const float* body_pos,
                          const float* body_vel, const float* normal, int32_t capacity) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "fem_set_soft_contacts: null handle");
    DeviceGuard g(H->device);
    return register_soft_contacts(H->h, count, particle, body_pos, body_vel, normal, capacity);
}

int fem_set_surface_contacts(FemHandle* H, int32_t body_count, const int32_t* body_start, const int32_t* body_size,
                             const int32_t* tri_offsets, const int32_t* triangles, float ke, float kd, const float* q,
                             void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "fem_set_surface_contacts: null handle");
    Handle& h = H->h;
    if (body_count < 0) return set_error(FEM_ERR_BAD_ARG, "fem_set_surface_contacts: negative body count");
    if (body_count > 0 && (!body_start || !body_size || !tri_offsets || !q || (tri_offsets[body_count] > 0 && !triangles)))
        return set_error(FEM_ERR_BAD_ARG, "fem_set_surface_contacts: null array");
    if (body_count > 0 && tri_offsets[0] != 0)
        return set_error(FEM_ERR_BAD_ARG, "fem_set_surface_contacts: triangle offsets must start at 0");
    for (int b = 0; b < body_count; ++b) {  // validate before replacing the current registration
        if (body_start[b] < 0 || body_size[b] < 0 || (int64_t)body_start[b] + body_size[b] > h.P)
            return set_error(FEM_ERR_BAD_ARG, "fem_set_surface_contacts: body ranges must lie inside the particles");
        if (tri_offsets[b + 1] < tri_offsets[b])
            return set_error(FEM_ERR_BAD_ARG, "fem_set_surface_contacts: triangle offsets must not decrease");
        for (int64_t k = 3 * (int64_t)tri_offsets[b]; k < 3 * (int64_t)tri_offsets[b + 1]; ++k)
            if (triangles[k] < 0 || triangles[k] >= body_size[b])
                return set_error(FEM_ERR_BAD_ARG,
                                 "fem_set_surface_contacts: surface triangle indices must be local to their body");
    }
    DeviceGuard g(H->device);
    h.sf_active = 0;
    h.sf_host_start.clear();
    h.sf_host_size.clear();
    h.sf_host_toff.clear();
    h.sf_host_tris.clear();
    if (body_count == 0 || h.P == 0) return FEM_OK;
    std::string why;
    const int code = fem::surface_register(h, body_count, body_start, body_size, tri_offsets, triangles, ke, kd, q,
                                           (cudaStream_t)stream, why);
    if (code == FEM_ERR_BAD_ARG) return set_error(code, "fem_set_surface_contacts: " + why);
    if (code != FEM_OK) return code;
    h.sf_host_start.assign(body_start, body_start + body_count);
    h.sf_host_size.assign(body_size, body_size + body_count);
    h.sf_host_toff.assign(tri_offsets, tri_offsets + body_count + 1);
    h.sf_host_tris.assign(triangles, triangles + 3 * (size_t)tri_offsets[body_count]);
    return FEM_OK;
}

int fem_update_surface_contacts(FemHandle* H, const float* q, void* stream) {
    if (H == nullptr || q == nullptr) return set_error(FEM_ERR_BAD_ARG, "fem_update_surface_contacts: null argument");
    DeviceGuard g(H->device);
    return cuda_status(fem::surface_refit(H->h, q, (cudaStream_t)stream), &H->h);
}

int fem_set_timing(FemHandle* H, int32_t enable) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    H->h.timing = enable != 0;
    return FEM_OK;
}

int fem_get_timing(FemHandle* H, double* pcg_ms_total, int64_t* launches) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    DeviceGuard g(H->device);
    double total = 0.0;
    int64_t n = 0;
    cudaError_t err = cudaSuccess;
    for (size_t k = 0; k + 1 < h.timing_events.size(); k += 2) {
        cudaEvent_t e0 = h.timing_events[k], e1 = h.timing_events[k + 1];
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
        ++n;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    h.timing_events.clear();
    if (pcg_ms_total) *pcg_ms_total = total;
    if (launches) *launches = n;
    return cuda_status(err, &h);
}

int fem_prepare_tet_updates(FemHandle* H, const FemDesc* d, int32_t original_node_count, void* stream) {
    if (H == nullptr || d == nullptr) return set_error(FEM_ERR_BAD_ARG, "fem_prepare_tet_updates: null handle or descriptor");
    Handle& h = H->h;
    const int N0 = original_node_count;
    if (h.streaming) return set_error(FEM_ERR_BAD_ARG, "Tetrahedral updates are already prepared");
    if (N0 < 1 || h.P % N0 != 0)
        return set_error(FEM_ERR_BAD_ARG, "The particle pool must contain whole copies of the original node set");
    if (h.T < 1 || h.H || h.S || h.Tri)
        return set_error(FEM_ERR_BAD_ARG, "Streaming assembly requires tetrahedral elements only");
    if (h.precond != FEM_PRECOND_BLOCK_DIAG)
        return set_error(FEM_ERR_BAD_ARG, "Streaming assembly requires the block_diag preconditioner");
    if (h.nfixed) return set_error(FEM_ERR_BAD_ARG, "Streaming topology is not supported with fixed_particle_indices");
    if (h.nscenes != 1) return set_error(FEM_ERR_UNSUPPORTED, "Streaming assembly supports one scene");
    if (d->particle_count != h.P || d->tet_count != h.T || d->hex_count || d->spring_count || d->tri_count)
        return set_error(FEM_ERR_BAD_ARG, "the descriptor must describe the solver's model");
    std::vector<std::vector<int>> cand;
    std::string why;
    int code = fem::streaming_candidate(d, N0, cand, why);
    if (code != FEM_OK) return set_error(code, why);
    DeviceGuard g(H->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_status(e, &h);
    FemDesc nd = *d;
    nd.dt = h.dt;
    nd.tolerance = h.tol;
    nd.maxiter = h.maxiter;
    nd.velocity_increment = h.dv_owned ? nullptr : h.dv;
    FemHandle* fresh = nullptr;
    code = fem::create_handle(&nd, &cand, &fresh);
    if (code != FEM_OK) return code;
    Handle& n = fresh->h;
    n.wait_limit_ns = h.wait_limit_ns;
    n.spmv_unroll = h.spmv_unroll;
    n.l2_resident_bytes = h.l2_resident_bytes;
    n.pcg_threads = h.pcg_threads;
    n.grid_cap = h.grid_cap;
    n.timing = h.timing;
    n.mu_scale = h.mu_scale;
    n.balance = h.balance;
    n.split_headroom = h.split_headroom;
    n.tail_prefetch = h.tail_prefetch;
    n.compact_cols = h.compact_cols;
    n.resident_pref = h.resident_pref;
    n.cg_variant = h.cg_variant;
    n.operator_batch = h.operator_batch;
    n.operator_stage = h.operator_stage;
    n.cta_speed = h.cta_speed;  // speeds belong to CTA indices, so they carry over to the new split
    code = register_soft_contacts(n, h.sc_count, h.sc_particle, h.sc_pos, h.sc_vel, h.sc_normal, h.sc_cap);
    if (code == FEM_OK) code = configure_launch(n);
    if (code == FEM_OK && !h.sf_host_start.empty()) code = carry_surfaces(h, n, h.rest);
    if (code == FEM_OK) {
        std::vector<int> diag(h.P);
        for (int r = 0; r < h.P; ++r) {
            const auto& c = cand[r];
            const int k = (int)(std::lower_bound(c.begin(), c.end(), r) - c.begin());
            diag[r] = (n.host_slice_ptr[r / fem::kSlice] + k) * fem::kSlice + (r % fem::kSlice);
        }
        code = cuda_status(fem::streaming_allocate(n, N0, diag), &n);
    }
    if (code != FEM_OK) {
        fem_destroy(fresh);
        return code;
    }
    std::swap(H->h, fresh->h);
    fresh->device = H->device;
    fem_destroy(fresh);
    // assemble at the construction positions with the identity lineage (streaming.py:515-516)
    FemTopologyUpdate u;
    code = fem::streaming_update(H->h, d, H->h.rest, nullptr, &u, (cudaStream_t)stream, why);
    if (code == FEM_ERR_BAD_ARG) return set_error(code, why);
    return code;
}

int fem_update_tet_topology(FemHandle* H, const FemDesc* d, float* q, float dt, const int32_t* element_sources,
                            FemTopologyUpdate* update, void* stream) {
    if (H == nullptr || d == nullptr || q == nullptr)
        return set_error(FEM_ERR_BAD_ARG, "fem_update_tet_topology: null handle, descriptor or positions");
    Handle& h = H->h;
    if (!h.streaming) return set_error(FEM_ERR_BAD_ARG, "Prepare tetrahedral updates before applying element sources");
    if (!(dt > 0.0f) || dt != h.dt)
        return set_error(FEM_ERR_BAD_ARG, "refresh_topology requires the currently assembled timestep");
    if (d->particle_count != h.P || d->tet_count != h.T || d->hex_count || d->spring_count || d->tri_count ||
        d->tet_indices == nullptr || d->tet_poses == nullptr || d->tet_materials == nullptr ||
        d->particle_mass == nullptr || d->particle_inv_mass == nullptr)
        return set_error(FEM_ERR_BAD_ARG, "topology updates must preserve the model's capacities");
    DeviceGuard g(H->device);
    std::string why;
    FemTopologyUpdate u;
    int code = fem::streaming_update(h, d, q, element_sources, update ? update : &u, (cudaStream_t)stream, why);
    if (code == FEM_ERR_BAD_ARG) return set_error(code, why);
    return code;
}

int fem_refresh_topology(FemHandle* H, const FemDesc* d, float* q, float dt, void* stream) {
    if (H == nullptr || d == nullptr || q == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle, descriptor or positions");
    if (H->h.streaming) return fem_update_tet_topology(H, d, q, dt, nullptr, nullptr, stream);
    Handle& h = H->h;
    if (!(dt > 0.0f) || !std::isfinite(dt)) return set_error(FEM_ERR_BAD_ARG, "dt must be finite and positive");
    if (dt != h.dt) return set_error(FEM_ERR_BAD_ARG, "refresh_topology requires the currently assembled timestep");
    if (h.precond != FEM_PRECOND_BLOCK_DIAG)
        return set_error(FEM_ERR_BAD_ARG, "persistent topology updates require the block_diag preconditioner");
    if (d->particle_count != h.P || d->tet_count != h.T || d->hex_count != h.H || d->spring_count != h.S ||
        d->tri_count != h.Tri || std::max(1, d->scene_count) != h.nscenes || d->fixed_count != h.nfixed)
        return set_error(FEM_ERR_BAD_ARG, "topology updates must preserve the model's capacities");
    DeviceGuard g(H->device);
    cudaError_t e = cudaDeviceSynchronize();  // nothing may still use the storage being replaced
    if (e != cudaSuccess) return cuda_status(e, &h);
    FemDesc nd = *d;
    nd.dt = dt;
    nd.tolerance = h.tol;
    nd.maxiter = h.maxiter;
    nd.velocity_increment = h.dv_owned ? nullptr : h.dv;
    FemHandle* fresh = nullptr;
    int code = fem_create(&nd, &fresh);
    if (code != FEM_OK) return code;
    Handle& n = fresh->h;
    n.wait_limit_ns = h.wait_limit_ns;
    n.spmv_unroll = h.spmv_unroll;
    n.l2_resident_bytes = h.l2_resident_bytes;
    n.pcg_threads = h.pcg_threads;
    n.grid_cap = h.grid_cap;
    n.timing = h.timing;
    n.mu_scale = h.mu_scale;
    n.balance = h.balance;
    n.split_headroom = h.split_headroom;
    n.tail_prefetch = h.tail_prefetch;
    n.compact_cols = h.compact_cols;
    n.resident_pref = h.resident_pref;
    n.cg_variant = h.cg_variant;
    n.operator_batch = h.operator_batch;
    n.operator_stage = h.operator_stage;
    n.cta_speed = h.cta_speed;  // speeds belong to CTA indices, so they carry over to the new split
    code = register_soft_contacts(n, h.sc_count, h.sc_particle, h.sc_pos, h.sc_vel, h.sc_normal, h.sc_cap);
    if (code == FEM_OK) code = configure_launch(n);
    if (code == FEM_OK && !h.sf_host_start.empty()) code = carry_surfaces(h, n, q);
    if (code != FEM_OK) {
        fem_destroy(fresh);
        return code;
    }
    std::swap(H->h, fresh->h);
    fresh->device = H->device;
    fem_destroy(fresh);  // frees the previous storage
    return fem_refresh_tangent(H, q, dt, stream);
}

int fem_refresh_tangent(FemHandle* H, float* q, float dt, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    if (!(dt > 0.0f) || !std::isfinite(dt)) return set_error(FEM_ERR_BAD_ARG, "refresh_tangent dt must be finite and positive");
    if (h.P == 0) {
        h.dt = dt;
        return FEM_OK;
    }
    if (q == nullptr) return set_error(FEM_ERR_BAD_ARG, "null positions");
    if (h.streaming && dt != h.dt)
        return set_error(FEM_ERR_BAD_ARG, "Streaming tangent refresh requires the construction timestep");
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = cudaSuccess;
    if (dt != h.dt) {  // solver.py:816-822: rebuild the dt-dependent blocks, clear the warm start
        err = cudaMemsetAsync(h.dv, 0, sizeof(float) * 3 * (size_t)h.P, s);
        if (err == cudaSuccess) err = fem::launch_constant_blocks(h, dt, s);
    }
    if (err == cudaSuccess) err = fem::launch_node_prepare(h, q, nullptr, true, false, false, s);
    if (err == cudaSuccess) err = fem::launch_element_tangent(h, dt, s);
    if (err == cudaSuccess) err = fem::launch_gather(h, s);
    if (err == cudaSuccess && h.streaming)  // the linearisation the next topology update compares against
        err = cudaMemcpyAsync(h.lin_q, q, sizeof(float) * 3 * (size_t)h.P, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && h.tangent_refreshes == 0)  // the first refresh refits the surfaces (solver.py:824-827, 669-670)
        err = fem::surface_refit(h, q, s);
    if (err == cudaSuccess) {
        h.dt = dt;
        h.tangent_refreshes += 1;
    }
    return cuda_status(err, &h);
}

int fem_rebuild_element_blocks(FemHandle* H, float* q, float dt, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    if (!(dt > 0.0f) || !std::isfinite(dt)) return set_error(FEM_ERR_BAD_ARG, "dt must be finite and positive");
    if (h.P == 0) return FEM_OK;
    if (q == nullptr) return set_error(FEM_ERR_BAD_ARG, "null positions");
    if (h.streaming) return fem_refresh_tangent(H, q, dt, stream);  // solver.py:672-674
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = fem::launch_node_prepare(h, q, nullptr, true, false, false, s);
    if (err == cudaSuccess) err = fem::launch_element_tangent(h, dt, s);
    if (err == cudaSuccess) err = fem::launch_gather(h, s);
    if (err == cudaSuccess) err = fem::surface_refit(h, q, s);  // solver.py:669-670
    return cuda_status(err, &h);
}

int fem_refresh_preconditioner(FemHandle* H, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    DeviceGuard g(H->device);
    // The inverse blocks are written by the assembly epilogue; re-running the
    // gather refreshes them in place from the current triplet values.
    return cuda_status(fem::launch_gather(H->h, (cudaStream_t)stream), &H->h);
}

int fem_set_tolerance(FemHandle* H, float tolerance) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    if (!(tolerance > 0.0f) || !std::isfinite(tolerance))
        return set_error(FEM_ERR_BAD_ARG, "linear_solver_tolerance must be finite and positive");
    H->h.tol = tolerance;
    return FEM_OK;
}

int fem_set_tuning(FemHandle* H, int32_t key, int64_t value) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    DeviceGuard g(H->device);
    if (key == FEM_TUNE_SPMV_UNROLL) {
        if (value != 1 && value != 2 && value != 4) return set_error(FEM_ERR_BAD_ARG, "unroll must be 1, 2 or 4");
        h.spmv_unroll = (int)value;
    } else if (key == FEM_TUNE_L2_RESIDENT_BYTES) {
        if (value < -2) return set_error(FEM_ERR_BAD_ARG, "resident bytes must be >= -2");
        h.l2_resident_bytes = value;
    } else if (key == FEM_TUNE_CTA_THREADS) {
        if (value != 0 && value != 256 && value != 512 && value != 1024)
            return set_error(FEM_ERR_BAD_ARG, "CTA threads must be 0 (automatic), 256, 512 or 1024");
        h.pcg_threads = (int)value;
    } else if (key == FEM_TUNE_GRID_CAP) {
        if (value < 0 || value > (1 << 20)) return set_error(FEM_ERR_BAD_ARG, "grid cap must be in [0, 2^20]");
        h.grid_cap = (int)value;
    } else if (key == FEM_TUNE_RESIDENT_LAYOUT) {
        if (value < -1 || value > 2) return set_error(FEM_ERR_BAD_ARG, "resident layout must be -1, 0, 1 or 2");
        h.resident_pref = (int)value;
    } else if (key == FEM_TUNE_COMPACT_COLUMNS) {
        if (value < -1 || value > 2) return set_error(FEM_ERR_BAD_ARG, "compact columns must be -1, 0, 1 or 2");
        h.compact_cols = (int)value;
    } else if (key == FEM_TUNE_OPERATOR_BATCH) {
        if (value != 2 && value != 4) return set_error(FEM_ERR_BAD_ARG, "operator batch must be 2 or 4");
        h.operator_batch = (int)value;
        return FEM_OK;  // fem_apply_operator only: no PCG launch tables to rebuild
    } else if (key == FEM_TUNE_OPERATOR_STAGE) {
        if (value != 0 && value != 4 && value != 8) return set_error(FEM_ERR_BAD_ARG, "operator stage must be 0, 4 or 8");
        h.operator_stage = (int)value;
        return FEM_OK;
    } else if (key == FEM_TUNE_CG_VARIANT) {
        if (value != 0 && value != 1) return set_error(FEM_ERR_BAD_ARG, "CG variant must be 0 or 1");
        h.cg_variant = (int)value;
    } else if (key == FEM_TUNE_TAIL_PREFETCH) {
        if (value < 0 || value > 100) return set_error(FEM_ERR_BAD_ARG, "tail prefetch must be 0..100 percent");
        h.tail_prefetch = (int)value;
        return FEM_OK;
    } else if (key == FEM_TUNE_SPLIT_HEADROOM) {
        if (value < 0 || value > 50) return set_error(FEM_ERR_BAD_ARG, "split headroom must be 0..50 percent");
        h.split_headroom = (int)value;
    } else if (key == FEM_TUNE_BALANCE) {
        if (value != 0 && value != 1) return set_error(FEM_ERR_BAD_ARG, "balance must be 0 or 1");
        h.balance = (int)value;
        h.cta_speed.clear();
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_status(e, &h);
        int code = configure_launch(h);
        if (code == FEM_OK && h.balance) code = calibrate_balance(h);
        return code;
    } else {
        return set_error(FEM_ERR_BAD_ARG, "unknown tuning key");
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_status(e, &h);
    return configure_launch(h);
}

int fem_get_tuning(FemHandle* H, int32_t key, int64_t* value) {
    if (H == nullptr || value == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle or output");
    Handle& h = H->h;
    switch (key) {
        case FEM_TUNE_SPMV_UNROLL: *value = h.spmv_unroll; return FEM_OK;
        case FEM_TUNE_L2_RESIDENT_BYTES: *value = h.l2_resident_bytes; return FEM_OK;
        case FEM_TUNE_RESIDENT_SLICES: *value = h.resident_slices; return FEM_OK;
        case FEM_TUNE_GRID: *value = h.grid; return FEM_OK;
        case FEM_TUNE_CTA_THREADS: *value = h.pcg_threads_used; return FEM_OK;
        case FEM_TUNE_GRID_CAP: *value = h.grid_cap; return FEM_OK;
        case FEM_TUNE_RESIDENT_STATE: *value = h.resident; return FEM_OK;
        case FEM_TUNE_BALANCE: *value = h.balance; return FEM_OK;
        case FEM_TUNE_RESIDENT_LAYOUT: *value = h.resident_pref; return FEM_OK;
        case FEM_TUNE_SPLIT_HEADROOM: *value = h.split_headroom; return FEM_OK;
        case FEM_TUNE_TAIL_PREFETCH: *value = h.tail_prefetch; return FEM_OK;
        case FEM_TUNE_COMPACT_COLUMNS: *value = column_mode(h); return FEM_OK;
        case FEM_TUNE_UNIFORM_COLUMN_BLOCKS: *value = column_mode(h) == 2 ? h.uniform_blocks : 0; return FEM_OK;
        case FEM_TUNE_CG_VARIANT: *value = h.cg_variant; return FEM_OK;
        case FEM_TUNE_OPERATOR_BATCH: *value = h.operator_batch; return FEM_OK;
        case FEM_TUNE_OPERATOR_STAGE: *value = h.operator_stage; return FEM_OK;
        default: return set_error(FEM_ERR_BAD_ARG, "unknown tuning key");
    }
}

int fem_set_wait_limit(FemHandle* H, int64_t nanoseconds) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    if (nanoseconds < 0) return set_error(FEM_ERR_BAD_ARG, "wait limit must be non-negative");
    H->h.wait_limit_ns = nanoseconds;
    return FEM_OK;
}

int fem_set_maxiter(FemHandle* H, int32_t maxiter) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    if (maxiter < 0) return set_error(FEM_ERR_BAD_ARG, "linear_solver_maxiter must be non-negative");
    H->h.maxiter = maxiter;
    return FEM_OK;
}

int fem_reset(FemHandle* H, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = cudaSuccess;
    if (h.P > 0) err = cudaMemsetAsync(h.dv, 0, sizeof(float) * 3 * (size_t)h.P, s);
    if (err == cudaSuccess && h.status) err = cudaMemsetAsync(h.status, 0, sizeof(int), s);
    return cuda_status(err, &h);
}

float* fem_velocity_increment_ptr(FemHandle* H) { return H ? H->h.dv : nullptr; }
int fem_get_solve_residuals(FemHandle* H, float* residuals, int32_t reset, void* stream) {
    if (H == nullptr || residuals == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle or output");
    Handle& h = H->h;
    residuals[0] = residuals[1] = 0.0f;
    if (h.P == 0) return FEM_OK;
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = cudaStreamSynchronize(s);
    if (err == cudaSuccess) err = cudaMemcpy(residuals, h.resid_max, 2 * sizeof(float), cudaMemcpyDeviceToHost);
    if (err == cudaSuccess && reset) err = cudaMemsetAsync(h.resid_max, 0, 2 * sizeof(float), s);
    return cuda_status(err, &h);
}


int fem_get_stats(FemHandle* H, FemStats* stats, int32_t* scene_iterations, void* stream) {
    if (H == nullptr || stats == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle or stats");
    Handle& h = H->h;
    DeviceGuard g(H->device);
    std::memset(stats, 0, sizeof(FemStats));
    stats->scene_count = h.nscenes;
    if (h.P == 0) return FEM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return cuda_status(err, &h);
    std::vector<fem::SceneStats> sc(h.nscenes);
    std::vector<long long> cum(h.nscenes);
    int status = 0;
    err = cudaMemcpy(sc.data(), h.scene_stats, sizeof(fem::SceneStats) * sc.size(), cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(&status, h.status, sizeof(int), cudaMemcpyDeviceToHost);
    if (err == cudaSuccess)
        err = cudaMemcpy(cum.data(), h.cum_iters, sizeof(long long) * cum.size(), cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_status(err, &h);
    stats->status = status;
    stats->total_iterations = 0;
    for (long long c : cum) stats->total_iterations += c;
    stats->max_iterations = 0;
    stats->min_iterations = sc.empty() ? 0 : INT32_MAX;
    float worst = 0.0f;
    for (int k = 0; k < h.nscenes; ++k) {
        stats->max_iterations = std::max(stats->max_iterations, sc[k].iterations);
        stats->min_iterations = std::min(stats->min_iterations, sc[k].iterations);
        float rel = sc[k].bb > 0.0f ? std::sqrt(sc[k].rr / sc[k].bb) : 0.0f;
        worst = std::max(worst, rel);
        if (!sc[k].converged) stats->unconverged_scenes++;
        if (scene_iterations) scene_iterations[k] = sc[k].iterations;
    }
    stats->max_relative_residual = worst;
    if (status & fem::kStatusTimeout) return FEM_ERR_TIMEOUT;
    if (status & fem::kStatusNonFinite) return FEM_ERR_NON_FINITE;
    return FEM_OK;
}

int fem_eval_forces(FemHandle* H, const float* q, const float* v, const float* activations, const float* gravity,
                    int32_t terms, float* out, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    if (!q || !v || !out) return set_error(FEM_ERR_BAD_ARG, "null pointer");
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = fem::launch_node_prepare(h, const_cast<float*>(q), const_cast<float*>(v), false, true, false, s);
    if (err == cudaSuccess) err = fem::launch_element_forces(h, activations, s);
    if (err == cudaSuccess) err = fem::launch_node_forces(h, nullptr, gravity, 1.0f, terms, false, out, s);
    return cuda_status(err, &h);
}

int fem_matrix_info(FemHandle* H, int64_t* nnzb, int64_t* triplet_count, int64_t* stored_blocks) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    if (nnzb) *nnzb = H->h.nnzb;
    if (triplet_count) *triplet_count = H->h.ntrip;
    if (stored_blocks) *stored_blocks = H->h.nsell;
    return FEM_OK;
}

int fem_export_bsr(FemHandle* H, int32_t* offsets, int32_t* columns, float* values, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = cudaSuccess;
    if (offsets && h.P > 0)
        err = cudaMemcpyAsync(offsets, h.bsr_offsets, sizeof(int) * (h.P + 1), cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && columns && h.nnzb > 0)
        err = cudaMemcpyAsync(columns, h.bsr_columns, sizeof(int) * h.nnzb, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && values) err = fem::launch_export_bsr(h, values, s);
    return cuda_status(err, &h);
}

int fem_export_preconditioner(FemHandle* H, float* inverse_blocks, void* stream) {
    if (H == nullptr || inverse_blocks == nullptr) return set_error(FEM_ERR_BAD_ARG, "null pointer");
    Handle& h = H->h;
    DeviceGuard g(H->device);
    if (h.P == 0) return FEM_OK;
    return cuda_status(cudaMemcpyAsync(inverse_blocks, h.minv, sizeof(float) * 9 * (size_t)h.P,
                                       cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
                       &h);
}

int fem_export_triplets(FemHandle* H, int32_t* rows, int32_t* columns, float* values, void* stream) {
    if (H == nullptr) return set_error(FEM_ERR_BAD_ARG, "null handle");
    Handle& h = H->h;
    DeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = cudaSuccess;
    if (rows && h.ntrip)
        err = cudaMemcpyAsync(rows, h.trip_rows, sizeof(int) * h.ntrip, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && columns && h.ntrip)
        err = cudaMemcpyAsync(columns, h.trip_cols, sizeof(int) * h.ntrip, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && values) err = fem::launch_export_triplets(h, values, s);
    return cuda_status(err, &h);
}

}  // extern "C"
