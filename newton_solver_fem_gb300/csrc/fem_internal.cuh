// Internal state of a FemHandle and the launchers shared between translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "fem_gb300.h"

namespace fem {

constexpr int kSlice = 32;          // rows per SELL slice (one warp, thread per row)
constexpr int kPcgMaxThreads = 1024;  // largest persistent PCG block (the launch bound)
constexpr unsigned kFixedBit = 0x80000000u;  // row_info: fixed-node flag; low bits = row length

// Device-side status bits (FemStats.status).
constexpr int kStatusTimeout = 1 << 2;
constexpr int kStatusNonFinite = 1 << 1;

// Triplet blocks (the reference layout [P | 2S | 3Tri | 16T | 64H]) stored in three
// planes, the same split as the SELL matrix: block i is (a[i], b[i], c[i]) =
// ((a00 a01 a02 a10), (a11 a12 a20 a21), a22), so that a block is written and
// read with two aligned 16-byte accesses and one 4-byte access.
struct TripletPlanes {
    float4* a = nullptr;
    float4* b = nullptr;
    float* c = nullptr;
};

#ifdef __CUDACC__
__device__ __forceinline__ void store_block(const TripletPlanes& t, int64_t i, const float* v) {
    t.a[i] = make_float4(v[0], v[1], v[2], v[3]);
    t.b[i] = make_float4(v[4], v[5], v[6], v[7]);
    t.c[i] = v[8];
}
#endif

// Per-scene persistent solver statistics written by the PCG epilogue.
struct SceneStats {
    int iterations;
    float rr;
    float bb;
    int converged;
};

// Everything a PCG launch needs (plain pointers, passed by value).
struct PcgArgs {
    // SELL-32 matrix: entry e = (slice_ptr[sl] + k) * 32 + lane
    const float4* __restrict__ valA;  // (a00 a01 a02 a10)
    const float4* __restrict__ valB;  // (a11 a12 a20 a21)
    const float* __restrict__ valC;   // a22
    const int* __restrict__ scol;     // block column
    const short* __restrict__ dcol;   // block column - row (when every offset fits 16 bits), or null
    const unsigned long long* __restrict__ slice_kmask;  // [nslices] slots k < 64 with one offset for the slice
    const short* __restrict__ slice_kval;                // [nslices * 64] that offset
    const int* __restrict__ slice_ptr;   // [nslices+1]
    const int2* __restrict__ slice_meta; // [nslices] (first row, row count)
    const int* __restrict__ slice_scene; // [nslices]
    const unsigned* __restrict__ row_info;  // [P] length | kFixedBit
    const float* __restrict__ minv;  // [P*9]
    int nslices;
    int slices_per_cta;  // L: the most slices any CTA owns (shared-memory sizing)
    const int* __restrict__ cta_slice0;  // [grid+1] CTA c's positions in cta_list: [cta_slice0[c], cta_slice0[c+1])
    unsigned long long* cta_time;        // [2*grid] SpMV-phase ns and iterations per CTA, or null
    int tail_prefetch;                   // prefetch a last round keeping at most this % of the warps busy (0 = off)
    // segment tables for deterministic per-scene reductions
    const int* __restrict__ cta_seg_base;     // [grid+1] CTA c's segments are [cta_seg_base[c], cta_seg_base[c+1])
    const int* __restrict__ seg_start;        // [nseg] a segment's first position in its CTA's slice list
    const int* __restrict__ seg_pos;          // [nseg] its slot in the segment buffer (scene-major)
    const int* __restrict__ cta_list;         // [nslices] CTA c owns slices cta_list[cta_slice0[c] .. cta_slice0[c+1])
    int contiguous;                           // every CTA's list is a contiguous run of slices
    const int* __restrict__ scene_seg0;       // [S+1]
    int nscenes;
    float* seg_part;  // [2][nseg * 3], alternating between consecutive reductions
    int nseg;
    // node data
    const float4* __restrict__ v4;     // packed velocity (fixed zeroed)
    const float4* __restrict__ q4;     // packed positions (fixed restored)
    const float* __restrict__ rest;    // [P*3] anchors
    const int* __restrict__ spring_ptr;   // node -> incident springs [P+1]
    const int* __restrict__ spring_ent;   // 2*s + endpoint
    const int* __restrict__ spring_idx;   // [2S]
    const float* __restrict__ spring_kd;  // [S]
    float* f_ws;       // [P*3] in: h*sum f, out: final rhs
    float* dv;         // [P*3] warm start in, velocity increment out
    float* q_out;      // [P*3]
    float* v_out;      // [P*3]
    // CG vectors.  z and the search direction p of a node share one 32-byte
    // record (zp[2i] = z_i, zp[2i+1] = p_i) so that a gathered column costs one
    // sector; two record buffers alternate between iterations.
    float4* x;
    float4* r;
    float4* zp0;
    float4* zp1;
    float4* stage;   // [2P] (p_i, y_i) handed from phase A to phase B when not staged in shared memory
    int stage_smem;  // 1: the staging lives in the CTA's shared memory
    int resident;    // rows' state in shared memory: 0 none, 1 x/r/z (x/r/p/s/w in the single-reduction
                     // variant), 2 the same and the inverse diagonal blocks
    // single-reduction variant: records (u, Mw, Ms) per node as 3 float4 in two alternating buffers,
    // own-row p, s, w in global memory when not resident
    float4* rec0;
    float4* rec1;
    float4* p4;
    float4* s4;
    float4* w4;
    // control
    unsigned* barrier;
    int* status;
    SceneStats* scene_stats;
    long long* cum_iters;  // [S] CG iterations summed over launches
    float* resid_max;      // [2] running max of the final relative residual: [0] step mode, [1] solve mode
    int maxiter;
    float tol;
    float dt;
    long long limit_ns;  // give up a barrier wait after this many ns
    int write_state;  // 1: integrate state (step); 0: solve only
    int resident_slices;  // slices [0, resident_slices) are loaded with the L2 evict_last policy
    const float* solve_rhs;  // non-null: solve A x = solve_rhs (no predictor), x -> dv
    int solve_warm;          // solve mode: start from the packed x (else from zero)
};

struct Handle {
    // sizes
    int P = 0, T = 0, H = 0, S = 0, Tri = 0, nfixed = 0, nscenes = 1;
    int64_t ntrip = 0, nnzb = 0, nsell = 0;
    int nslices = 0;
    // options
    float dt = 0.f, min_stretch = 0.f, max_stretch = 0.f;
    int has_ground = 0;
    float ground[4] = {0, 0, 1, 0};
    float gke = 0, gkd = 0, gkf = 0, gmu = 0, linear_damping = 0;
    float gravity_init[3] = {0, 0, 0};
    int enable_act = 0, precond = 0, maxiter = 50;
    float tol = 1e-2f;
    long long wait_limit_ns = 2000000000LL;
    int spmv_unroll = 4;          // block columns in flight per thread in the PCG SpMV (1, 2 or 4)
    int64_t l2_resident_bytes = -2;  // matrix bytes loaded evict_last (-1: 60% of L2; -2: all if it fits there, else 0)
    int pcg_threads = 0;             // threads per PCG CTA (256, 512, 1024; 0 = chosen from the problem size)
    int balance = 0;                 // 1: slices split by calibrated per-CTA speed (FEM_TUNE_BALANCE)
    int split_headroom = 0;          // % more slices per CTA than the even share a calibrated split may use
    int tail_prefetch = 50;          // FEM_TUNE_TAIL_PREFETCH (percent of warps busy in the last round)
    int resident_pref = -1;          // resident row-state layout: -1 automatic, 0 none, 1 x/r/z, 2 x/r/z + inverse
    int cg_variant = 0;              // FEM_TUNE_CG_VARIANT: 0 standard CG, 1 single-reduction (Chronopoulos-Gear)
    int operator_batch = 2;          // FEM_TUNE_OPERATOR_BATCH: block columns in flight per thread in fem_apply_operator
    int operator_stage = 4;          // FEM_TUNE_OPERATOR_STAGE: 0 direct loads, else block columns per bulk copy
    std::vector<double> cta_speed;   // calibrated SpMV speed per CTA index (cost units per ns)
    std::vector<int64_t> host_slice_cost;  // stored blocks + 4 per live row, per slice
    std::vector<int> host_cta_slice0;      // the partition in use: CTA c owns host_cta_list[cta_slice0[c] ..)
    std::vector<int> host_cta_list;        // slice indices, ascending within each CTA
    int* cta_slice0 = nullptr;
    int* cta_list = nullptr;
    int cta_contiguous = 1;                // every CTA owns a contiguous run of slices
    unsigned long long* cta_time = nullptr;  // set only while calibrating
    int pcg_threads_used = 0;        // the CTA size of the current configuration
    int grid_cap = 0;                // upper bound on the PCG grid (0: co-residency limit only)
    int resident_slices = 0;
    bool tangent_prepared = false;
    int tangent_refreshes = 0;       // fem_refresh_tangent calls (the first one refits the surfaces)
    // node data
    float* rest = nullptr;
    float* mass = nullptr;
    float* inv_mass = nullptr;
    float* radius = nullptr;
    int* flags = nullptr;
    int* fixed_idx = nullptr;
    unsigned char* fixed_mask = nullptr;
    float* gravity_dev = nullptr;  // construction gravity (used when the step passes none)
    // elements
    int4* tet_idx = nullptr;
    float* tet_pose = nullptr;  // [T*9]
    float* tet_mat = nullptr;   // [T*3]
    int* hex_idx = nullptr;     // [H*8]
    float* hex_invJ = nullptr;  // [H*72]
    float* hex_detw = nullptr;  // [H*8]
    float* hex_mat = nullptr;   // [H*3]
    const float* mu_scale = nullptr;  // optional caller-owned per-tet shear scale [T]
    float4* elem_grad = nullptr;      // adjoint scratch [2 * (4T + 8H + 3Tri)], allocated on first VJP
    float* roll_f = nullptr;          // rollout scratch [3P]: the substep right-hand side (first rollout call)
    float* adj_vt = nullptr;          // adjoint scratch [3P]: the adjoint solve's right-hand side
    float* adj_x = nullptr;           // adjoint scratch [3P]: the adjoint solution when the caller keeps none
    int* tri_idx = nullptr;     // [Tri*3]
    float4* tri_pose = nullptr; // [Tri] (Dm00, Dm01, Dm10, Dm11)
    float* tri_mat = nullptr;   // [Tri*5] (ke, ka, kd, drag, lift)
    int* spring_idx = nullptr;  // [2S]
    float* spring_rest = nullptr;
    float* spring_ke = nullptr;
    float* spring_kd = nullptr;
    float* spring_dir = nullptr;  // [3S] rest directions when the bend torque is active, else null
    float torque_ke = 0.f, torque_kd = 0.f;
    // particle-particle contact (hash grid rebuilt at every force evaluation)
    int pcontact = 0;
    float pke = 0.f, pkd = 0.f, pkf = 0.f, pmu = 0.f, pcoh = 0.f, pmaxr = 0.f;
    int grid_dim = 0;              // buckets per axis (power of two); grid_dim^3 buckets
    int* grid_count = nullptr;     // [nb] particles per bucket (zero between evaluations)
    int* grid_start = nullptr;     // [nb+1] exclusive scan of grid_count
    int* grid_part = nullptr;      // scan block sums
    int* grid_items = nullptr;     // [P] particle ids by bucket, ascending within a bucket
    int* cell_of = nullptr;        // [P] bucket of each active particle or -1
    float4* pforce = nullptr;      // [P] particle-contact force
    // soft-rigid contacts (caller-owned list registered per step)
    float ske = 0.f, skd = 0.f, skf = 0.f, smu = 0.f;
    const int* sc_count = nullptr;
    const int* sc_particle = nullptr;
    const float* sc_pos = nullptr;
    const float* sc_vel = nullptr;
    const float* sc_normal = nullptr;
    int sc_cap = 0, sc_alloc = 0;
    int* sc_head = nullptr;        // [P] first contact of each particle's list or -1
    int* sc_next = nullptr;        // [sc_alloc]
    float4* sc_force = nullptr;    // [sc_alloc]
    // incidence
    int* node_elem_ptr = nullptr;  // [P+1]
    int* node_elem_ent = nullptr;  // element-force slots
    int* node_spring_ptr = nullptr;
    int* node_spring_ent = nullptr;
    // streaming Tet4 assembly (reserved candidate pattern, topology updates on the device)
    int streaming = 0;
    int orig_nodes = 0;            // nodes per copy of the original node set
    int4* st_idx = nullptr;        // [T] staged connectivity of an update
    float* st_pose = nullptr;      // [9T]
    float* st_mat = nullptr;       // [3T]
    int4* old_idx = nullptr;       // [T] published connectivity of the previous update
    float* old_pose = nullptr;     // [9T]
    float* old_mat = nullptr;      // [3T]
    int* old_active = nullptr;     // [T]
    float* lin_q = nullptr;        // [3P] positions of the last linearisation
    int* st_active = nullptr;      // [T]
    int* st_same = nullptr;        // [T] corners equal to the source's
    int* st_slot = nullptr;        // [16T] SELL entry of each block of an active element
    int* topo_winner = nullptr;    // [T] per source: lowest element keeping its topology
    int* reuse_src = nullptr;      // [T] per source: numeric block reusable
    int* topo_src = nullptr;       // [T] per source: topology kept
    int* touched = nullptr;        // [P]
    int* counters = nullptr;       // [8] error code and lineage counters
    int* entry_count = nullptr;    // [nsell] zero between updates
    int* node_count = nullptr;     // [P] zero between updates
    int* diag_entry = nullptr;     // [P] SELL entry of each diagonal block
    int* scan_part = nullptr;
    // soft-body surface contacts (per-body triangle surfaces with BVHs)
    int sf_active = 0, sf_nbody = 0, sf_ntri = 0, sf_nsurf = 0, sf_nnode = 0, sf_nleaf = 0, sf_nvert = 0;
    float sf_ke = 0.f, sf_kd = 0.f;
    int4* sf_tri = nullptr;        // [ntri] (i, j, k, body), leaf order
    int4* sf_node = nullptr;       // [nnode] (left, right, first tri, tri count)
    int* sf_parent = nullptr;      // [nnode]
    int* sf_root = nullptr;        // [nbody] root node or -1
    float* sf_max_dist = nullptr;  // [nbody] rest bounding-box diagonal
    int* sf_surf = nullptr;        // [nsurf] surface particles
    int* sf_surf_body = nullptr;   // [nsurf]
    int* sf_adj = nullptr;         // [3 ntri] triangle across each edge or -1
    int* sf_vslot = nullptr;       // [P] mesh-vertex slot or -1
    int* sf_verts = nullptr;       // [nvert] mesh vertices
    int* sf_vt_ptr = nullptr;      // [nvert+1] incident (triangle, corner) lists
    int* sf_vt = nullptr;
    int* sf_leaves = nullptr;      // [nleaf]
    int* sf_arrivals = nullptr;    // [nnode] refit counters
    float4 *sf_x = nullptr, *sf_force = nullptr;  // [P] refit positions, surface force
    float4 *sf_fn = nullptr, *sf_en = nullptr, *sf_vn = nullptr, *sf_lo = nullptr, *sf_hi = nullptr;
    std::vector<int> sf_host_start, sf_host_size, sf_host_toff, sf_host_tris;  // registration (re-applied on rebuild)
    // per-step scratch
    float4* elem_force = nullptr;  // [4T + 8H + 3Tri]
    float4* q4 = nullptr;
    float4* v4 = nullptr;
    // assembly
    TripletPlanes trip;           // [ntrip] blocks
    int* sell_slot = nullptr;     // [nsell] canonical slot or -1
    int* sell_cptr = nullptr;     // [nsell+1] contributor range of each SELL entry
    int* sell_contrib = nullptr;  // triplet ids, ascending within each entry
    int* bsr_offsets = nullptr;   // [P+1]
    int* bsr_columns = nullptr;   // [nnzb]
    int* slot_sell = nullptr;     // [nnzb] canonical slot -> SELL entry
    int* trip_rows = nullptr;     // [ntrip] (export only)
    int* trip_cols = nullptr;
    // SELL matrix
    float4* valA = nullptr;
    float4* valB = nullptr;
    float* valC = nullptr;
    int* scol = nullptr;
    short* dcol = nullptr;  // [nsell] column - row when every offset fits 16 bits (the PCG reads these), else null
    int compact_cols = -1;  // FEM_TUNE_COMPACT_COLUMNS: 0 scol, 1 dcol, 2 dcol + uniform slots, -1 automatic
    int64_t uniform_blocks = 0;  // stored blocks in uniform slots (FEM_TUNE_UNIFORM_COLUMN_BLOCKS)
    unsigned long long* slice_kmask = nullptr;  // [nslices] bit k: every row of the slice has the same dcol at k
    unsigned* fixcol = nullptr;  // [nsell / 32] per (slice, k): lanes whose column at k is a fixed node (null: none)
    short* slice_kval = nullptr;                // [nslices * 64] that dcol
    int* slice_ptr = nullptr;
    int2* slice_meta = nullptr;
    int* slice_scene = nullptr;
    int* sell_row = nullptr;  // [nsell] row of entry (or -1 for lanes past the slice)
    unsigned* row_info = nullptr;
    float* minv = nullptr;  // [P*9]
    // CG
    float4 *x = nullptr, *r = nullptr;
    float4 *zp0 = nullptr, *zp1 = nullptr;  // [2P] each: (z_i, p_i) records
    float4* stage = nullptr;                // [2P] (p_i, y_i) phase A -> phase B staging
    // single-reduction variant (launch allocations): (u, Mw, Ms) records in two alternating buffers
    // [3P] each, and the own-row p, s, w when they are not resident in shared memory [P] each
    float4 *rec0 = nullptr, *rec1 = nullptr, *p4 = nullptr, *s4 = nullptr, *w4 = nullptr;
    int stage_smem = 0;
    int resident = 0;                       // row state resident in shared memory (see PcgArgs)
    float* dv = nullptr;
    bool dv_owned = true;
    // reductions / control
    int grid = 0;
    size_t pcg_smem = 0;
    int slices_per_cta = 0;
    int* cta_seg_base = nullptr;  // [grid+1]
    int* seg_start = nullptr;     // [nseg]
    int* seg_pos = nullptr;       // [nseg]
    int* scene_seg0 = nullptr;
    int nseg = 0;
    float* seg_part = nullptr;
    unsigned* barrier = nullptr;
    int* status = nullptr;
    SceneStats* scene_stats = nullptr;
    long long* cum_iters = nullptr;
    float* resid_max = nullptr;  // [2] largest relative residual of step-mode / solve-mode solves since the last read
    // optional timing of PCG launches (eager launches only)
    bool timing = false;
    std::vector<cudaEvent_t> timing_events;  // start/end pairs
    std::vector<void*> allocations;
    std::vector<void*> launch_allocations;  // segment tables, rebuilt on a tuning change
    std::vector<int> host_slice_scene;
    std::vector<int> host_slice_ptr;
    std::string last_error;
};

// Handle construction (fem_api.cu); `candidate` reserves per-row sorted columns (streaming Tet4 assembly).
int create_handle(const FemDesc* d, const std::vector<std::vector<int>>* candidate, FemHandle** out);

// Status reporting shared by every entry point: the message is what
// fem_status_string returns for the code (fem_api.cu).
int report(int code, const char* message);
int report_cuda(cudaError_t err);

// dN_a/dxi at the 8 Gauss points (host copy, filled as the reference computes it)
void fill_hex_reference_table(float table[8][8][3]);
void upload_hex_reference_table();          // fem_elements.cu copy
void upload_hex_reference_table_adjoint();  // fem_adjoint.cu copy

// --- launchers (fem_elements.cu) ---
cudaError_t launch_node_prepare(Handle& h, float* q, float* v, bool restore_fixed, bool pack_v, bool pack_x,
                                cudaStream_t s);
cudaError_t launch_element_forces(Handle& h, const float* activations, cudaStream_t s);
cudaError_t launch_node_forces(Handle& h, const float* ext, const float* gravity, float dt, int terms, bool scale_by_dt,
                               float* out, cudaStream_t s);
cudaError_t launch_constant_blocks(Handle& h, float dt, cudaStream_t s);
// The column storage a handle's PCG launches read (FEM_TUNE_COMPACT_COLUMNS):
// 0 without 16-bit offsets; automatic (-1) reads shared slot offsets once per
// slice (2) when the matrix streams from DRAM, and per row (1) when all of it is
// kept in L2, where the saved bytes no longer pay for the extra instructions.
inline int column_mode(const Handle& h) {
    if (h.dcol == nullptr || h.compact_cols == 0) return 0;
    if (h.compact_cols == 1 || h.slice_kmask == nullptr) return 1;
    if (h.compact_cols == 2) return 2;
    return h.resident_slices < h.nslices ? 2 : 1;
}

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }
// first triplet of the Tet4 region: [P | 2S | 3Tri | 16T | 64H]
inline int64_t tet_triplet_offset(const Handle& h) {
    return (int64_t)h.P + 2 * (int64_t)h.S + 3 * (int64_t)h.Tri;
}
// --- streaming Tet4 assembly (fem_streaming.cu) ---
int streaming_candidate(const FemDesc* d, int original_nodes, std::vector<std::vector<int>>& rows, std::string& why);
cudaError_t streaming_allocate(Handle& h, int original_nodes, const std::vector<int>& diag_entry);
int streaming_update(Handle& h, const FemDesc* d, const float* q, const int* sources, FemTopologyUpdate* out,
                     cudaStream_t s, std::string& why);
// --- soft-body surface contacts (fem_surface.cu) ---
int surface_register(Handle& h, int nbody, const int32_t* body_start, const int32_t* body_size,
                     const int32_t* tri_offsets, const int32_t* triangles, float ke, float kd, const float* q,
                     cudaStream_t s, std::string& why);
cudaError_t surface_refit(Handle& h, const float* q, cudaStream_t s);
cudaError_t launch_surface_contacts(Handle& h, cudaStream_t s);  // into h.sf_force
// --- launchers (fem_contacts.cu) ---
int particle_grid_dim(int P);
// Exclusive scan of count[0, n) into start[0, n] (start[n] = total); part holds
// scan_partial_count(n) ints.
int scan_partial_count(int64_t n);
cudaError_t launch_exclusive_scan(const int* count, int* start, int n, int* part, cudaStream_t s);
cudaError_t launch_particle_contacts(Handle& h, cudaStream_t s);  // grid build + per-particle force into h.pforce
cudaError_t launch_soft_contacts(Handle& h, cudaStream_t s);      // per-contact force + per-particle lists
cudaError_t launch_element_tangent(Handle& h, float dt, cudaStream_t s);
// --- launchers (fem_assembly.cu) ---
cudaError_t launch_gather(Handle& h, cudaStream_t s);
cudaError_t launch_export_bsr(Handle& h, float* values, cudaStream_t s);
cudaError_t launch_export_triplets(Handle& h, float* values, cudaStream_t s);
// --- launchers (fem_pcg.cu) ---
// Lets `kernel` launch with up to `bytes` of dynamic shared memory on the current device.  The limit is
// a property of the kernel, shared by every handle that launches it, so it is only ever raised: setting
// it for one handle never invalidates another handle's launch (or a captured graph's).
cudaError_t allow_dynamic_smem(const void* kernel, size_t bytes);
cudaError_t pcg_configure(Handle& h);
// Step mode (solve_rhs == nullptr): predictor, normalised PCG from the dv warm start, integration.
// Solve mode: A x = solve_rhs from zero (projected at fixed rows), x written to x_out.
// Solve mode with solve_warm: start from the packed h.x instead of zero (normalised like step mode).
cudaError_t launch_pcg(Handle& h, float dt, int write_state, float* q_out, float* v_out, float* f_ws, cudaStream_t s,
                       const float* solve_rhs = nullptr, float* x_out = nullptr, float tol = -1.0f,
                       int maxiter = -1, bool solve_warm = false);

}  // namespace fem

// The opaque handle of the C ABI.
struct FemHandle {
    fem::Handle h;
    int device = 0;
};
