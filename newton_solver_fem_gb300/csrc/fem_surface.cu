// Soft-body surface contacts (reference soft_surface_contacts.py;
// SolverFEM.set_soft_surface_contacts solver.py:510-540, evaluated last in
// _accumulate_forces solver.py:551-589).
//
// Every registered body has a triangle surface over its own particles.  Each
// surface vertex of a body is queried against every other body's surface for
// the closest point within that body's rest bounding-box diagonal; the
// inside/outside sign comes from the angle-weighted pseudonormal of the
// closest feature (face, edge or vertex) -- the sign test of Baerentzen and
// Aanaes for closed meshes -- and a penetration r - signed distance > 0 gives
// the penalty force n (ke pen - kd min(v.n, 0)).
//
// The surfaces use the positions of their last refit (registration, the first
// tangent refresh, every element-block rebuild and explicit updates), as the
// reference's refitted BVH meshes do, while the queried vertices use the
// current positions.  Per body, a BVH over the triangles is built once on the
// host by median splits of the registration positions; a refit recomputes
// face normals, pseudonormals and node bounds on the device (bounds bottom-up:
// the second child to arrive at a node writes the union, which does not depend
// on the arrival order).  A query traverses nearest child first with an
// explicit stack; ties keep the first triangle found, in that fixed order.
#include <algorithm>
#include <climits>
#include <cmath>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "fem_internal.cuh"
#include "fem_math.cuh"

namespace fem {

namespace {

constexpr int kLeafTris = 4;
constexpr int kStackDepth = 64;

// Closest point on triangle (a, b, c) to p (the Voronoi-region method of
// Ericson, Real-Time Collision Detection 5.1.5).  feature: 0 face, 1..3 edge
// ab, bc, ca, 4..6 vertex a, b, c.
__device__ float3 closest_on_triangle(float3 p, float3 a, float3 b, float3 c, int& feature) {
    const float3 ab = b - a, ac = c - a, ap = p - a;
    const float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) {
        feature = 4;
        return a;
    }
    const float3 bp = p - b;
    const float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) {
        feature = 5;
        return b;
    }
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        feature = 1;
        return a + ab * (d1 / (d1 - d3));
    }
    const float3 cp = p - c;
    const float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) {
        feature = 6;
        return c;
    }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        feature = 3;
        return a + ac * (d2 / (d2 - d6));
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        feature = 2;
        return b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)));
    }
    feature = 0;
    const float denom = 1.0f / (va + vb + vc);
    return a + ab * (vb * denom) + ac * (vc * denom);
}

__device__ __forceinline__ float box_dist2(float3 p, float4 lo, float4 hi) {
    const float dx = fmaxf(fmaxf(lo.x - p.x, 0.0f), p.x - hi.x);
    const float dy = fmaxf(fmaxf(lo.y - p.y, 0.0f), p.y - hi.y);
    const float dz = fmaxf(fmaxf(lo.z - p.z, 0.0f), p.z - hi.z);
    return dx * dx + dy * dy + dz * dz;
}

__global__ void surface_snapshot_kernel(int n, const int* __restrict__ verts, const float* __restrict__ q,
                                        float4* __restrict__ x) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int v = verts[k];
    x[v] = make_float4(q[3 * v], q[3 * v + 1], q[3 * v + 2], 0.0f);
}

__global__ void surface_face_kernel(int nt, const int4* __restrict__ tri, const float4* __restrict__ x,
                                    float4* __restrict__ fn) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int4 f = tri[t];
    const float3 a = xyz(x[f.x]), b = xyz(x[f.y]), c = xyz(x[f.z]);
    float3 n = cross3(b - a, c - a);
    const float l = len3(n);
    n = l > 0.0f ? n * (1.0f / l) : f3(0.f, 0.f, 0.f);
    fn[t] = f4(n);
}

__device__ __forceinline__ float corner_angle(float3 p, float3 q, float3 r) {
    const float3 u = q - p, v = r - p;
    const float lu = len3(u), lv = len3(v);
    if (lu <= 0.0f || lv <= 0.0f) return 0.0f;
    return acosf(fminf(fmaxf(dot3(u, v) / (lu * lv), -1.0f), 1.0f));
}

// Angle-weighted vertex pseudonormals (incident triangles in ascending order)
// and edge pseudonormals (the two adjacent face normals).
__global__ void surface_pseudonormal_kernel(int nv, const int* __restrict__ vt_ptr,
                                            const int* __restrict__ vt, const int4* __restrict__ tri,
                                            const float4* __restrict__ x, const float4* __restrict__ fn,
                                            float4* __restrict__ vn) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nv) return;
    float3 s = f3(0.f, 0.f, 0.f);
    for (int e = vt_ptr[k]; e < vt_ptr[k + 1]; ++e) {
        const int t = vt[e] >> 2, c = vt[e] & 3;
        const int4 f = tri[t];
        const float3 a = xyz(x[f.x]), b = xyz(x[f.y]), d = xyz(x[f.z]);
        const float ang = c == 0 ? corner_angle(a, b, d) : (c == 1 ? corner_angle(b, d, a) : corner_angle(d, a, b));
        s = s + xyz(fn[t]) * ang;
    }
    vn[k] = f4(s);
}

__global__ void surface_edge_kernel(int nt, const int* __restrict__ adj, const float4* __restrict__ fn,
                                    float4* __restrict__ en) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 3 * nt) return;
    const int t = k / 3, o = adj[k];
    float3 n = xyz(fn[t]);
    if (o >= 0) n = n + xyz(fn[o]);
    en[k] = f4(n);
}

// Bottom-up bounds: each leaf boxes its triangles and climbs; at every node
// the first arriving child stops and the second writes the union.
__global__ void surface_refit_kernel(int nleaf, const int* __restrict__ leaves, const int4* __restrict__ node,
                                     const int* __restrict__ parent, const int4* __restrict__ tri,
                                     const float4* __restrict__ x, float4* lo, float4* hi, int* arrivals) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nleaf) return;
    int nd = leaves[k];
    const int4 leaf = node[nd];
    float3 l = f3(INFINITY, INFINITY, INFINITY), h = f3(-INFINITY, -INFINITY, -INFINITY);
    for (int t = leaf.z; t < leaf.z + leaf.w; ++t) {
        const int4 f = tri[t];
        const int vs[3] = {f.x, f.y, f.z};
        for (int c = 0; c < 3; ++c) {
            const float3 p = xyz(x[vs[c]]);
            l = f3(fminf(l.x, p.x), fminf(l.y, p.y), fminf(l.z, p.z));
            h = f3(fmaxf(h.x, p.x), fmaxf(h.y, p.y), fmaxf(h.z, p.z));
        }
    }
    lo[nd] = f4(l);
    hi[nd] = f4(h);
    for (;;) {
        const int pa = parent[nd];
        if (pa < 0) return;
        __threadfence();
        if (atomicAdd(arrivals + pa, 1) == 0) return;  // the sibling finishes this node
        __threadfence();
        const int4 in = node[pa];
        const float4 la = __ldcg(lo + in.x), ha = __ldcg(hi + in.x), lb = __ldcg(lo + in.y), hb = __ldcg(hi + in.y);
        lo[pa] = make_float4(fminf(la.x, lb.x), fminf(la.y, lb.y), fminf(la.z, lb.z), 0.0f);
        hi[pa] = make_float4(fmaxf(ha.x, hb.x), fmaxf(ha.y, hb.y), fmaxf(ha.z, hb.z), 0.0f);
        nd = pa;
    }
}

struct SurfaceQueryArgs {
    int nsurf, nbody;
    const int* surf;
    const int* surf_body;
    const int* root;
    const float* max_dist;
    const int4* node;
    const float4* lo;
    const float4* hi;
    const int4* tri;
    const float4* x;      // positions of the last refit
    const float4* fn;
    const float4* en;
    const float4* vn;     // per mesh-vertex slot
    const int* vslot;     // [P] mesh-vertex slot of a particle, or -1
    const float4* q4;     // current positions
    const float4* v4;
    const float* radius;
    const int* flags;
    float ke, kd;
    float4* out;
};

__global__ void surface_query_kernel(SurfaceQueryArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nsurf) return;
    const int p = a.surf[k];
    float3 f = f3(0.f, 0.f, 0.f);
    if ((a.flags[p] & 1) != 0) {
        const float3 xp = xyz(a.q4[p]), vp = xyz(a.v4[p]);
        const float r = a.radius[p];
        const int mine = a.surf_body[k];
        for (int b = 0; b < a.nbody; ++b) {
            if (b == mine || a.root[b] < 0) continue;
            const float md = a.max_dist[b];
            float best2 = md * md;
            int best_t = -1, best_feat = 0;
            float3 best_c = f3(0.f, 0.f, 0.f);
            int stack[kStackDepth];
            int sp = 0;
            stack[sp++] = a.root[b];
            while (sp > 0) {
                const int nd = stack[--sp];
                if (box_dist2(xp, a.lo[nd], a.hi[nd]) >= best2) continue;
                const int4 n = a.node[nd];
                if (n.w > 0) {
                    for (int t = n.z; t < n.z + n.w; ++t) {
                        const int4 tr = a.tri[t];
                        int feat;
                        const float3 c = closest_on_triangle(xp, xyz(a.x[tr.x]), xyz(a.x[tr.y]), xyz(a.x[tr.z]), feat);
                        const float3 d = xp - c;
                        const float d2 = dot3(d, d);
                        if (d2 < best2) {
                            best2 = d2;
                            best_t = t;
                            best_feat = feat;
                            best_c = c;
                        }
                    }
                } else if (sp + 2 <= kStackDepth) {
                    // push the farther child first, so the nearer one is visited first
                    const float dl = box_dist2(xp, a.lo[n.x], a.hi[n.x]), dr = box_dist2(xp, a.lo[n.y], a.hi[n.y]);
                    if (dl <= dr) {
                        stack[sp++] = n.y;
                        stack[sp++] = n.x;
                    } else {
                        stack[sp++] = n.x;
                        stack[sp++] = n.y;
                    }
                }
            }
            if (best_t < 0) continue;
            const float3 diff = xp - best_c;
            const float raw = len3(diff);
            if (raw < 1.0e-8f) continue;
            float3 pn;
            if (best_feat == 0) {
                pn = xyz(a.fn[best_t]);
            } else if (best_feat <= 3) {
                pn = xyz(a.en[3 * best_t + best_feat - 1]);
            } else {
                const int4 tr = a.tri[best_t];
                const int v = best_feat == 4 ? tr.x : (best_feat == 5 ? tr.y : tr.z);
                pn = xyz(a.vn[a.vslot[v]]);
            }
            const float sign = dot3(diff, pn) >= 0.0f ? 1.0f : -1.0f;
            const float3 n = diff * (sign / raw);
            const float pen = r - raw * sign;
            if (!(pen > 0.0f)) continue;
            const float vn = dot3(vp, n);
            const float fn = a.ke * pen - a.kd * fminf(vn, 0.0f);
            f = f + n * fn;
        }
    }
    a.out[p] = make_float4(f.x, f.y, f.z, 0.0f);
}

template <class T>
T* upload_vec(Handle& h, const std::vector<T>& v, cudaError_t& e) {
    if (e != cudaSuccess) return nullptr;
    void* p = nullptr;
    e = cudaMalloc(&p, std::max<size_t>(1, v.size()) * sizeof(T));
    if (e != cudaSuccess) return nullptr;
    h.allocations.push_back(p);
    if (!v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return static_cast<T*>(p);
}

}  // namespace

// Registration: host-side BVHs, adjacency and incidence; device arrays; first refit at q.
int surface_register(Handle& h, int nbody, const int32_t* body_start, const int32_t* body_size,
                     const int32_t* tri_offsets, const int32_t* triangles, float ke, float kd, const float* q,
                     cudaStream_t s, std::string& why) {
    const int P = h.P;
    std::vector<float> host_q(3 * (size_t)P);
    cudaError_t e = cudaMemcpy(host_q.data(), q, sizeof(float) * host_q.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return report_cuda(e);
    std::vector<int4> tri;          // (i, j, k, body), global node ids, leaf order
    std::vector<int4> node;         // (left, right, first tri, tri count); leaf when count > 0
    std::vector<int> parent, root(nbody, -1), surf, surf_body;
    std::vector<float> max_dist(nbody, 0.0f);
    for (int b = 0; b < nbody; ++b) {
        const int start = body_start[b], size = body_size[b];
        if (start < 0 || size < 0 || start + size > P) {
            why = "surface body ranges must lie inside the particle array";
            return FEM_ERR_BAD_ARG;
        }
        const int t0 = tri_offsets[b], t1 = tri_offsets[b + 1];
        if (t1 < t0) {
            why = "surface triangle offsets must not decrease";
            return FEM_ERR_BAD_ARG;
        }
        if (t1 == t0) continue;  // a body without surface data is never queried (reference placeholder)
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = start; i < start + size; ++i)
            for (int c = 0; c < 3; ++c) {
                lo[c] = std::min(lo[c], host_q[3 * (size_t)i + c]);
                hi[c] = std::max(hi[c], host_q[3 * (size_t)i + c]);
            }
        max_dist[b] = size > 0 ? std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                           (hi[2] - lo[2]) * (hi[2] - lo[2]))
                               : 0.0f;
        std::vector<int4> bt;
        std::vector<int> verts;
        for (int t = t0; t < t1; ++t) {
            int g[3];
            for (int c = 0; c < 3; ++c) {
                const int l = triangles[3 * (size_t)t + c];
                if (l < 0 || l >= size) {
                    why = "surface triangle indices must be local to their body";
                    return FEM_ERR_BAD_ARG;
                }
                g[c] = start + l;
                verts.push_back(g[c]);
            }
            bt.push_back(make_int4(g[0], g[1], g[2], b));
        }
        std::sort(verts.begin(), verts.end());
        verts.erase(std::unique(verts.begin(), verts.end()), verts.end());
        for (int v : verts) {
            surf.push_back(v);
            surf_body.push_back(b);
        }
        // median-split BVH over centroids
        std::vector<float> cen(3 * bt.size());
        for (size_t t = 0; t < bt.size(); ++t)
            for (int c = 0; c < 3; ++c)
                cen[3 * t + c] = (host_q[3 * (size_t)bt[t].x + c] + host_q[3 * (size_t)bt[t].y + c] +
                                  host_q[3 * (size_t)bt[t].z + c]) / 3.0f;
        std::vector<int> order(bt.size());
        std::iota(order.begin(), order.end(), 0);
        const int base_tri = (int)tri.size();
        struct Item { int node, lo, hi; };
        root[b] = (int)node.size();
        node.push_back(make_int4(-1, -1, 0, 0));
        parent.push_back(-1);
        std::vector<Item> work{{root[b], 0, (int)bt.size()}};
        while (!work.empty()) {
            const Item it = work.back();
            work.pop_back();
            if (it.hi - it.lo <= kLeafTris) {
                node[it.node] = make_int4(-1, -1, base_tri + it.lo, it.hi - it.lo);
                continue;
            }
            float cl[3] = {INFINITY, INFINITY, INFINITY}, ch[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int k = it.lo; k < it.hi; ++k)
                for (int c = 0; c < 3; ++c) {
                    cl[c] = std::min(cl[c], cen[3 * order[k] + c]);
                    ch[c] = std::max(ch[c], cen[3 * order[k] + c]);
                }
            int axis = 0;
            for (int c = 1; c < 3; ++c)
                if (ch[c] - cl[c] > ch[axis] - cl[axis]) axis = c;
            const int mid = (it.lo + it.hi) / 2;
            std::nth_element(order.begin() + it.lo, order.begin() + mid, order.begin() + it.hi, [&](int x, int y) {
                return cen[3 * x + axis] < cen[3 * y + axis] || (cen[3 * x + axis] == cen[3 * y + axis] && x < y);
            });
            const int left = (int)node.size(), right = left + 1;
            node.push_back(make_int4(-1, -1, 0, 0));
            node.push_back(make_int4(-1, -1, 0, 0));
            parent.push_back(it.node);
            parent.push_back(it.node);
            node[it.node] = make_int4(left, right, 0, 0);
            work.push_back({right, mid, it.hi});
            work.push_back({left, it.lo, mid});
        }
        for (int k : order) tri.push_back(bt[k]);
    }
    const int nt = (int)tri.size();
    // edge adjacency (within a body) and vertex incidence
    std::vector<int> adj(3 * (size_t)nt, -1);
    {
        std::map<std::pair<int, int>, std::vector<int>> edges;
        for (int t = 0; t < nt; ++t) {
            const int v[3] = {tri[t].x, tri[t].y, tri[t].z};
            for (int k = 0; k < 3; ++k) {
                const int a = v[k], b = v[(k + 1) % 3];
                edges[{std::min(a, b), std::max(a, b)}].push_back(3 * t + k);
            }
        }
        for (auto& kv : edges)
            for (int x : kv.second)
                for (int y : kv.second)
                    if (x != y && adj[x] < 0) adj[x] = y / 3;
    }
    std::vector<int> vslot(P, -1), mesh_verts;
    for (int t = 0; t < nt; ++t)
        for (int v : {tri[t].x, tri[t].y, tri[t].z})
            if (vslot[v] < 0) {
                vslot[v] = 0;
                mesh_verts.push_back(v);
            }
    std::sort(mesh_verts.begin(), mesh_verts.end());
    for (size_t k = 0; k < mesh_verts.size(); ++k) vslot[mesh_verts[k]] = (int)k;
    std::vector<int> vt_ptr(mesh_verts.size() + 1, 0), vt;
    for (int t = 0; t < nt; ++t)
        for (int v : {tri[t].x, tri[t].y, tri[t].z}) vt_ptr[vslot[v] + 1]++;
    for (size_t k = 0; k < mesh_verts.size(); ++k) vt_ptr[k + 1] += vt_ptr[k];
    vt.resize(vt_ptr.back());
    {
        std::vector<int> pos(vt_ptr.begin(), vt_ptr.end() - 1);
        for (int t = 0; t < nt; ++t) {
            const int v[3] = {tri[t].x, tri[t].y, tri[t].z};
            for (int c = 0; c < 3; ++c) vt[pos[vslot[v[c]]]++] = 4 * t + c;
        }
    }
    std::vector<int> leaves;
    for (size_t n = 0; n < node.size(); ++n)
        if (node[n].w > 0) leaves.push_back((int)n);

    h.sf_nbody = nbody;
    h.sf_ntri = nt;
    h.sf_nsurf = (int)surf.size();
    h.sf_nnode = (int)node.size();
    h.sf_nleaf = (int)leaves.size();
    h.sf_nvert = (int)mesh_verts.size();
    h.sf_ke = ke;
    h.sf_kd = kd;
    e = cudaSuccess;
    h.sf_tri = upload_vec(h, tri, e);
    h.sf_node = upload_vec(h, node, e);
    h.sf_parent = upload_vec(h, parent, e);
    h.sf_root = upload_vec(h, root, e);
    h.sf_max_dist = upload_vec(h, max_dist, e);
    h.sf_surf = upload_vec(h, surf, e);
    h.sf_surf_body = upload_vec(h, surf_body, e);
    h.sf_adj = upload_vec(h, adj, e);
    h.sf_vslot = upload_vec(h, vslot, e);
    h.sf_verts = upload_vec(h, mesh_verts, e);
    h.sf_vt_ptr = upload_vec(h, vt_ptr, e);
    h.sf_vt = upload_vec(h, vt, e);
    h.sf_leaves = upload_vec(h, leaves, e);
    std::vector<float4> zero4(std::max<size_t>(1, (size_t)P), make_float4(0.f, 0.f, 0.f, 0.f));
    h.sf_x = upload_vec(h, zero4, e);
    h.sf_force = upload_vec(h, zero4, e);
    h.sf_fn = upload_vec(h, std::vector<float4>(std::max(1, nt)), e);
    h.sf_en = upload_vec(h, std::vector<float4>(3 * (size_t)std::max(1, nt)), e);
    h.sf_vn = upload_vec(h, std::vector<float4>(std::max<size_t>(1, mesh_verts.size())), e);
    h.sf_lo = upload_vec(h, std::vector<float4>(std::max<size_t>(1, node.size())), e);
    h.sf_hi = upload_vec(h, std::vector<float4>(std::max<size_t>(1, node.size())), e);
    h.sf_arrivals = upload_vec(h, std::vector<int>(std::max<size_t>(1, node.size()), 0), e);
    if (e != cudaSuccess) return report_cuda(e);
    h.sf_active = 1;
    return report_cuda(surface_refit(h, q, s));
}

cudaError_t surface_refit(Handle& h, const float* q, cudaStream_t s) {
    if (!h.sf_active || h.sf_ntri == 0) return cudaSuccess;
    surface_snapshot_kernel<<<blocks_for(h.sf_nvert, 256), 256, 0, s>>>(h.sf_nvert, h.sf_verts, q, h.sf_x);
    surface_face_kernel<<<blocks_for(h.sf_ntri, 256), 256, 0, s>>>(h.sf_ntri, h.sf_tri, h.sf_x, h.sf_fn);
    surface_pseudonormal_kernel<<<blocks_for(h.sf_nvert, 256), 256, 0, s>>>(h.sf_nvert, h.sf_vt_ptr, h.sf_vt, h.sf_tri,
                                                                            h.sf_x, h.sf_fn, h.sf_vn);
    surface_edge_kernel<<<blocks_for(3 * (int64_t)h.sf_ntri, 256), 256, 0, s>>>(h.sf_ntri, h.sf_adj, h.sf_fn, h.sf_en);
    cudaError_t e = cudaMemsetAsync(h.sf_arrivals, 0, sizeof(int) * (size_t)h.sf_nnode, s);
    if (e != cudaSuccess) return e;
    surface_refit_kernel<<<blocks_for(h.sf_nleaf, 128), 128, 0, s>>>(h.sf_nleaf, h.sf_leaves, h.sf_node, h.sf_parent,
                                                                    h.sf_tri, h.sf_x, h.sf_lo, h.sf_hi,
                                                                    h.sf_arrivals);
    return cudaGetLastError();
}

cudaError_t launch_surface_contacts(Handle& h, cudaStream_t s) {
    if (!h.sf_active || h.sf_nsurf == 0 || h.sf_nbody < 2) return cudaSuccess;
    SurfaceQueryArgs a;
    a.nsurf = h.sf_nsurf;
    a.nbody = h.sf_nbody;
    a.surf = h.sf_surf;
    a.surf_body = h.sf_surf_body;
    a.root = h.sf_root;
    a.max_dist = h.sf_max_dist;
    a.node = h.sf_node;
    a.lo = h.sf_lo;
    a.hi = h.sf_hi;
    a.tri = h.sf_tri;
    a.x = h.sf_x;
    a.fn = h.sf_fn;
    a.en = h.sf_en;
    a.vn = h.sf_vn;
    a.vslot = h.sf_vslot;
    a.q4 = h.q4;
    a.v4 = h.v4;
    a.radius = h.radius;
    a.flags = h.flags;
    a.ke = h.sf_ke;
    a.kd = h.sf_kd;
    a.out = h.sf_force;
    surface_query_kernel<<<blocks_for(h.sf_nsurf, 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fem
