// refharness.cpp — runs the VISGSim reference's own CUDA kernels (refkern.cubin,
// built from the reference sources by oracle/build.py) so that the library can be
// checked against them on the same inputs.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/ and the golden-fixture script, never by
// the library.
//
// The device work is entirely the reference's: compute_morton_bbox and init_nodes
// (bvh.cu:71-79,184-195), processInternalNode and calculateBoudingBox
// (cudaBRT.cu:120-206), verlet (verlet.cu:129-161, which calls D_BVH::intersect and
// Primitive::d_intersect).  This file restates only BVHAccel's host orchestration
// (bvh.cu:239-297; the class itself is tied to the OBJ/GL Mesh) and the Simulator's
// buffer handling (simulation.cu:54-100,182-194,243-257), with two documented
// reference-compatible choices: the root box is the exact union of all expanded
// triangle boxes (computed from the boxes compute_morton_bbox returns) instead of
// get_bb's partial union, and the host sort is stable (ties by triangle index).
// Physics constants are written into the module's __constant__ variables
// (verlet.cu:13-21); the spring damping kd = -0.5 is fixed in the kernel.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/visg_sim.h"

namespace {

// device-side layouts of the reference types (glm::vec3 = 3 floats)
struct RVec3 { float x, y, z; };
struct RBBox { RVec3 max, min, extent; };  // bbox.h:8-10 member order
struct RPrim { const void* vertices; const RVec3* d_vertices; uint32_t v0, v1, v2; };  // primitive.h:35-39
struct RNode { uint32_t counter; RBBox bbox; int childA, childB, parent, idx; };       // cudaBRT.h:34-115
struct RDBVH { const RPrim* d_primitives; RNode* d_leaf_nodes; RNode* d_internal_nodes; };  // cudaBRT.h:117-144
struct RSpring { int end; float original; };
static_assert(sizeof(RBBox) == 36, "BBox layout");
static_assert(sizeof(RNode) == 56, "BRTreeNode layout");
static_assert(sizeof(RPrim) == 32, "Primitive layout");

std::string g_msg;
CUmodule g_mod = nullptr;
CUfunction f_verlet, f_morton, f_init_nodes, f_internal, f_refit;
CUfunction f_vbo_pos = nullptr, f_face_normal = nullptr, f_vbo_normal = nullptr;

int fail(const std::string& m) {
    g_msg = m;
    return -1;
}
#define RT(x)                                                                                 \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess) return fail(std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define DRV(x)                                                       \
    do {                                                             \
        CUresult r_ = (x);                                           \
        if (r_ != CUDA_SUCCESS) {                                    \
            const char* s_ = nullptr;                                \
            cuGetErrorString(r_, &s_);                               \
            return fail(std::string(#x) + ": " + (s_ ? s_ : "?"));   \
        }                                                            \
    } while (0)

RBBox identity() {
    RBBox b;
    b.max = {-100.0f, -100.0f, -100.0f};
    b.min = {100.0f, 100.0f, 100.0f};
    b.extent = {-200.0f, -200.0f, -200.0f};
    return b;
}
void expand(RBBox& a, const RBBox& b) {  // bbox.h:62-73
    a.min.x = std::fmin(a.min.x, b.min.x); a.min.y = std::fmin(a.min.y, b.min.y); a.min.z = std::fmin(a.min.z, b.min.z);
    a.max.x = std::fmax(a.max.x, b.max.x); a.max.y = std::fmax(a.max.y, b.max.y); a.max.z = std::fmax(a.max.z, b.max.z);
    a.extent.x = a.max.x - a.min.x; a.extent.y = a.max.y - a.min.y; a.extent.z = a.max.z - a.min.z;
}

int launch(CUfunction f, unsigned grid, unsigned block, void** args) {
    DRV(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr));
    RT(cudaDeviceSynchronize());
    return 0;
}

struct RefBvh {
    int T = 0, Tp = 0;
    RVec3* d_verts = nullptr;
    RPrim* d_prims = nullptr;  // sorted
    RNode* d_leaf = nullptr;
    RNode* d_int = nullptr;
    std::vector<uint32_t> codes;  // per triangle
    std::vector<RBBox> boxes;     // per triangle
    std::vector<uint32_t> sorted_codes;
    std::vector<int32_t> sorted_tris;
    RBBox root;
    void free_all() {
        cudaFree(d_verts); cudaFree(d_prims); cudaFree(d_leaf); cudaFree(d_int);
        d_verts = nullptr; d_prims = nullptr; d_leaf = nullptr; d_int = nullptr;
    }
    // BVHAccel::BVHAccel (bvh.cu:264-297) on vertices that are already extended
    int build(const float* xyz, int nv, const uint32_t* tris, int nt) {
        free_all();
        T = nt;
        if (nt < 2) return fail("refkern needs at least two triangles");
        RT(cudaMalloc(&d_verts, sizeof(RVec3) * nv));
        RT(cudaMemcpy(d_verts, xyz, sizeof(RVec3) * nv, cudaMemcpyHostToDevice));
        std::vector<RPrim> prims(nt);
        for (int t = 0; t < nt; ++t) prims[t] = RPrim{nullptr, d_verts, tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
        RPrim* d_tmp_prims = nullptr;
        uint32_t* d_codes = nullptr;
        RBBox* d_boxes = nullptr;
        RT(cudaMalloc(&d_tmp_prims, sizeof(RPrim) * nt));
        RT(cudaMalloc(&d_codes, 4 * nt));
        RT(cudaMalloc(&d_boxes, sizeof(RBBox) * nt));
        RT(cudaMemcpy(d_tmp_prims, prims.data(), sizeof(RPrim) * nt, cudaMemcpyHostToDevice));
        unsigned threads = std::min(512u, (unsigned)nt), blocks = (nt + threads - 1) / threads;
        // pass 1: the reference's expanded boxes; the exact root box is their union
        RBBox bb = identity();
        int n = nt;
        void* a1[] = {&n, &d_tmp_prims, &bb, &d_codes, &d_boxes};
        if (launch(f_morton, blocks, threads, a1)) return -1;
        boxes.resize(nt);
        RT(cudaMemcpy(boxes.data(), d_boxes, sizeof(RBBox) * nt, cudaMemcpyDeviceToHost));
        root = identity();
        for (auto& b : boxes) expand(root, b);
        // pass 2: Morton codes in that frame (compute_morton_bbox, bvh.cu:71-79)
        bb = root;
        void* a2[] = {&n, &d_tmp_prims, &bb, &d_codes, &d_boxes};
        if (launch(f_morton, blocks, threads, a2)) return -1;
        codes.resize(nt);
        RT(cudaMemcpy(codes.data(), d_codes, 4 * nt, cudaMemcpyDeviceToHost));
        RT(cudaMemcpy(boxes.data(), d_boxes, sizeof(RBBox) * nt, cudaMemcpyDeviceToHost));
        cudaFree(d_tmp_prims); cudaFree(d_codes); cudaFree(d_boxes);
        // indices_sort (stable) + remove_redundant + filter (Utilities.h:23-67)
        std::vector<int32_t> idx(nt);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return codes[a] < codes[b]; });
        sorted_codes.clear();
        sorted_tris.clear();
        for (int k = 0; k < nt; ++k)
            if (k == 0 || codes[idx[k]] != sorted_codes.back()) {
                sorted_codes.push_back(codes[idx[k]]);
                sorted_tris.push_back(idx[k]);
            }
        Tp = (int)sorted_codes.size();
        if (Tp < 2) return fail("refkern needs at least two distinct Morton codes");
        std::vector<RPrim> sp(Tp);
        std::vector<RBBox> sb(Tp);
        for (int i = 0; i < Tp; ++i) { sp[i] = prims[sorted_tris[i]]; sb[i] = boxes[sorted_tris[i]]; }
        // BVHAccel::init + build (bvh.cu:197-237)
        uint32_t* d_sc = nullptr;
        RBBox* d_sb = nullptr;
        RT(cudaMalloc(&d_prims, sizeof(RPrim) * Tp));
        RT(cudaMalloc(&d_sc, 4 * Tp));
        RT(cudaMalloc(&d_sb, sizeof(RBBox) * Tp));
        RT(cudaMemcpy(d_prims, sp.data(), sizeof(RPrim) * Tp, cudaMemcpyHostToDevice));
        RT(cudaMemcpy(d_sc, sorted_codes.data(), 4 * Tp, cudaMemcpyHostToDevice));
        RT(cudaMemcpy(d_sb, sb.data(), sizeof(RBBox) * Tp, cudaMemcpyHostToDevice));
        RT(cudaMalloc(&d_leaf, sizeof(RNode) * Tp));
        RT(cudaMalloc(&d_int, sizeof(RNode) * (Tp - 1)));
        unsigned nl = (unsigned)Tp, ni = (unsigned)(Tp - 1);
        void* a3[] = {&d_leaf, &nl};
        if (launch(f_init_nodes, (nl + 1023) / 1024, 1024, a3)) return -1;
        void* a4[] = {&d_int, &ni};
        if (launch(f_init_nodes, (ni + 1023) / 1024, 1024, a4)) return -1;
        int nint = Tp - 1, nleaf = Tp;
        void* a5[] = {&d_sc, &nint, &d_leaf, &d_int};
        if (launch(f_internal, (nint + 1023) / 1024, 1024, a5)) return -1;
        void* a6[] = {&d_sb, &nleaf, &d_leaf, &d_int};
        if (launch(f_refit, (nleaf + 1023) / 1024, 1024, a6)) return -1;
        cudaFree(d_sc);
        cudaFree(d_sb);
        return check_refit();
    }

    // calculateBoudingBox (cudaBRT.cu:166-206) reads a sibling's box after atomicInc
    // without a fence, so now and then an internal box misses part of a child (a
    // stale read).  Its definition, evaluated here on the host over the reference's
    // own links and leaf boxes: every internal box is the identity box expanded by
    // child A's box, then child B's, children first.  Boxes that differ are counted
    // in `stale`; with `repair` the defined boxes replace the raced ones on the
    // device, so that every other kernel of the reference runs on the tree its
    // refit defines.
    int64_t stale = 0;
    bool repair = false;
    int check_refit() {
        const int ni = Tp - 1;
        std::vector<RNode> leaf(Tp), in(ni);
        RT(cudaMemcpy(leaf.data(), d_leaf, sizeof(RNode) * Tp, cudaMemcpyDeviceToHost));
        RT(cudaMemcpy(in.data(), d_int, sizeof(RNode) * ni, cudaMemcpyDeviceToHost));
        std::vector<RBBox> def(ni);
        std::vector<char> done(ni, 0);
        std::vector<int> stack{0};
        auto box = [&](int c) -> const RBBox& { return c < 0 ? leaf[-c - 1].bbox : def[c - 1]; };
        while (!stack.empty()) {
            const int i = stack.back();
            const int ca = in[i].childA, cb = in[i].childB;
            if (ca == 0 || cb == 0 || ca > ni || cb > ni || ca < -Tp || cb < -Tp) return fail("refit check: bad link");
            bool ready = true;
            if (ca > 0 && !done[ca - 1]) { stack.push_back(ca - 1); ready = false; }
            if (cb > 0 && !done[cb - 1]) { stack.push_back(cb - 1); ready = false; }
            if (!ready) continue;
            stack.pop_back();
            RBBox b = identity();
            expand(b, box(ca));
            expand(b, box(cb));
            def[i] = b;
            done[i] = 1;
        }
        int64_t n_stale = 0;
        for (int i = 0; i < ni; ++i)
            if (std::memcmp(&def[i], &in[i].bbox, sizeof(RBBox)) != 0) {
                ++n_stale;
                in[i].bbox = def[i];
            }
        stale += n_stale;
        if (repair && n_stale) RT(cudaMemcpy(d_int, in.data(), sizeof(RNode) * ni, cudaMemcpyHostToDevice));
        return 0;
    }
};

struct RefSim {
    VisgParams p;
    int N = 0;
    RVec3 *x[2] = {nullptr, nullptr}, *xo[2] = {nullptr, nullptr}, *cf = nullptr;
    uint32_t *row_s = nullptr, *row_b = nullptr;
    RSpring *ent_s = nullptr, *ent_b = nullptr;
    int read = 0;
    RefBvh bvh;
    int nv = 0;
    std::vector<uint32_t> tris;
    ~RefSim() {
        for (int k = 0; k < 2; ++k) { cudaFree(x[k]); cudaFree(xo[k]); }
        cudaFree(cf); cudaFree(row_s); cudaFree(row_b); cudaFree(ent_s); cudaFree(ent_b);
        bvh.free_all();
    }
    int set_constants() {
        auto put = [&](const char* name, const void* v, size_t sz) -> int {
            CUdeviceptr d;
            size_t bytes;
            DRV(cuModuleGetGlobal(&d, &bytes, g_mod, name));
            if (bytes != sz) return fail(std::string("constant size mismatch: ") + name);
            DRV(cuMemcpyHtoD(d, v, sz));
            return 0;
        };
        double ks = p.list_k[0], kb = p.list_k[1];
        if (put("spring_structure", &ks, 8) || put("spring_bend", &kb, 8) || put("damp", &p.force_damping, 4) ||
            put("mass", &p.mass, 4) || put("dt", &p.dt, 4) || put("gravit_x", &p.gravity[0], 4) ||
            put("gravit_y", &p.gravity[1], 4) || put("gravit_z", &p.gravity[2], 4))
            return -1;
        return 0;
    }
    int body(const float* xyz, const float* nrm) {
        std::vector<float> v(xyz, xyz + 3 * (size_t)nv);
        if (nrm)  // Mesh::vertex_extend (Mesh.cpp:101-117)
            for (size_t i = 0; i < v.size(); ++i) v[i] = v[i] + p.thickness * nrm[i];
        return bvh.build(v.data(), nv, tris.data(), (int)tris.size() / 3);
    }
    int step() {  // Simulator::cuda_verlet + swap_buffer (simulation.cu:182-194,243-251)
        if (set_constants()) return -1;
        RDBVH d{bvh.d_prims, bvh.d_leaf, bvh.d_int};
        RVec3 *xi = x[read], *xoi = xo[read], *xout = x[read ^ 1], *xoout = xo[read ^ 1];
        unsigned n = (unsigned)N;
        void* a[] = {&xi, &xoi, &xout, &xoout, &row_s, &ent_s, &row_b, &ent_b, &d, &cf, &n};
        unsigned threads = std::min(512u, n), blocks = (n + threads - 1) / threads;
        if (launch(f_verlet, blocks, threads, a)) return -1;
        read ^= 1;
        return 0;
    }
};

int find_fn(const char* prefix, CUfunction* out) {
    unsigned cnt = 0;
    DRV(cuModuleGetFunctionCount(&cnt, g_mod));
    std::vector<CUfunction> fs(cnt);
    DRV(cuModuleEnumerateFunctions(fs.data(), cnt, g_mod));
    for (auto f : fs) {
        const char* name = nullptr;
        DRV(cuFuncGetName(&name, f));
        if (name && std::strncmp(name, prefix, std::strlen(prefix)) == 0) {
            *out = f;
            return 0;
        }
    }
    return fail(std::string("kernel not found: ") + prefix);
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_msg.c_str(); }

int ref_init(const char* cubin) {
    if (g_mod) return 0;
    RT(cudaFree(nullptr));  // primary context current on this thread
    DRV(cuModuleLoad(&g_mod, cubin));
    if (find_fn("_Z6verlet", &f_verlet) || find_fn("_Z19compute_morton_bbox", &f_morton) ||
        find_fn("_Z10init_nodes", &f_init_nodes) || find_fn("_Z19processInternalNode", &f_internal) ||
        find_fn("_Z19calculateBoudingBox", &f_refit))
        return -1;
    return 0;
}

// The output stage of Simulator::cuda_update_vbo (simulation.cu:196-231) with the
// reference's own kernels: update_vbo_pos on x (the positions after the step),
// compute_face_normal on x_prev (the positions the step started from), then
// compute_vbo_normal over the vertex -> face CSR that get_vertex_adjface
// (simulation.cu:152-180) builds; device buffers stand in for the GL buffers.
int ref_render(const float* x, const float* x_prev, int n, const uint32_t* faces, int nf, float* pos4, float* vn,
               float* fn) {
    if (!f_vbo_pos && (find_fn("_Z14update_vbo_pos", &f_vbo_pos) || find_fn("_Z19compute_face_normal", &f_face_normal) ||
                       find_fn("_Z18compute_vbo_normal", &f_vbo_normal)))
        return -1;
    std::vector<std::vector<uint32_t>> adj(n);
    for (int f = 0; f < nf; ++f)
        for (int j = 0; j < 3; ++j) adj[faces[3 * f + j]].push_back((uint32_t)f);
    std::vector<uint32_t> row, col;
    uint32_t start = 0;
    for (int i = 0; i < n; ++i) {
        row.push_back(start);
        start += (uint32_t)adj[i].size();
        for (uint32_t f : adj[i]) col.push_back(f);
    }
    row.push_back(start);
    float *dx, *dxp, *dpos, *dvn, *dfn;
    uint32_t *dfaces, *drow, *dcol;
    RT(cudaMalloc((void**)&dx, 12 * (size_t)n));
    RT(cudaMalloc((void**)&dxp, 12 * (size_t)n));
    RT(cudaMalloc((void**)&dpos, 16 * (size_t)n));
    RT(cudaMalloc((void**)&dvn, 12 * (size_t)n));
    RT(cudaMalloc((void**)&dfn, 12 * (size_t)nf + 12));
    RT(cudaMalloc((void**)&dfaces, 12 * (size_t)nf + 12));
    RT(cudaMalloc((void**)&drow, 4 * row.size()));
    RT(cudaMalloc((void**)&dcol, 4 * col.size() + 4));
    RT(cudaMemcpy(dx, x, 12 * (size_t)n, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dxp, x_prev, 12 * (size_t)n, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dfaces, faces, 12 * (size_t)nf, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(drow, row.data(), 4 * row.size(), cudaMemcpyHostToDevice));
    if (!col.empty()) RT(cudaMemcpy(dcol, col.data(), 4 * col.size(), cudaMemcpyHostToDevice));
    unsigned un = (unsigned)n, idx_size = 3u * (unsigned)nf;
    void* a1[] = {&dpos, &dx, &un};
    if (launch(f_vbo_pos, (un + 511) / 512, 512, a1)) return -1;
    void* a2[] = {&dxp, &dfaces, &idx_size, &dfn};
    if (nf > 0 && launch(f_face_normal, ((unsigned)nf + 511) / 512, 512, a2)) return -1;
    void* a3[] = {&dvn, &drow, &dcol, &dfn, &un};
    if (launch(f_vbo_normal, (un + 1023) / 1024, 1024, a3)) return -1;
    RT(cudaMemcpy(pos4, dpos, 16 * (size_t)n, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(vn, dvn, 12 * (size_t)n, cudaMemcpyDeviceToHost));
    if (nf > 0) RT(cudaMemcpy(fn, dfn, 12 * (size_t)nf, cudaMemcpyDeviceToHost));
    void* ps[] = {dx, dxp, dpos, dvn, dfn, dfaces, drow, dcol};
    for (void* q : ps) cudaFree(q);
    return 0;
}

// Two spring lists (structure, bend) as in the reference.  Pass body normals to
// apply the thickness push.  Returns NULL on failure (see ref_last_error).
void* ref_sim_create(const VisgParams* p, const float* xyz, int N, const uint32_t* row_s, const VisgSpring* ent_s,
                     const uint32_t* row_b, const VisgSpring* ent_b, const float* body, const float* nrm, int nv,
                     const uint32_t* tris, int nt) {
    auto* s = new RefSim();
    s->p = *p;
    s->N = N;
    s->nv = nv;
    s->tris.assign(tris, tris + 3 * (size_t)nt);
    auto fail_null = [&](cudaError_t e) -> void* {
        g_msg = cudaGetErrorString(e);
        delete s;
        return nullptr;
    };
    size_t vb = sizeof(RVec3) * N;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = cudaMalloc(&s->x[k], vb);
        if (e == cudaSuccess) e = cudaMalloc(&s->xo[k], vb);
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->cf, vb);
    if (e == cudaSuccess) e = cudaMemset(s->cf, 0, vb);
    if (e == cudaSuccess) e = cudaMemcpy(s->x[0], xyz, vb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->xo[0], xyz, vb, cudaMemcpyHostToDevice);
    uint32_t Es = row_s[N], Eb = row_b[N];
    if (e == cudaSuccess) e = cudaMalloc(&s->row_s, 4 * (N + 1));
    if (e == cudaSuccess) e = cudaMalloc(&s->row_b, 4 * (N + 1));
    if (e == cudaSuccess) e = cudaMalloc(&s->ent_s, 8 * (Es + 1));
    if (e == cudaSuccess) e = cudaMalloc(&s->ent_b, 8 * (Eb + 1));
    if (e == cudaSuccess) e = cudaMemcpy(s->row_s, row_s, 4 * (N + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->row_b, row_b, 4 * (N + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && Es) e = cudaMemcpy(s->ent_s, ent_s, 8 * Es, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && Eb) e = cudaMemcpy(s->ent_b, ent_b, 8 * Eb, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_null(e);
    if (s->body(body, nrm)) {
        delete s;
        return nullptr;
    }
    return s;
}

void ref_sim_destroy(void* h) { delete (RefSim*)h; }
int ref_sim_step(void* h, int n) {
    for (int k = 0; k < n; ++k)
        if (((RefSim*)h)->step()) return -1;
    return 0;
}
int ref_sim_update_body(void* h, const float* xyz, const float* nrm) { return ((RefSim*)h)->body(xyz, nrm); }

// Simulator::update_vertex (simulation.cu:253-257)
int ref_sim_set_vertex(void* h, int idx, const float* v) {
    auto* s = (RefSim*)h;
    RT(cudaMemcpy(&s->x[s->read][idx], v, 12, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(&s->xo[s->read][idx], v, 12, cudaMemcpyHostToDevice));
    return 0;
}

int ref_sim_get_state(void* h, float* x, float* xo, float* n) {
    auto* s = (RefSim*)h;
    size_t vb = sizeof(RVec3) * s->N;
    if (x) RT(cudaMemcpy(x, s->x[s->read], vb, cudaMemcpyDeviceToHost));
    if (xo) RT(cudaMemcpy(xo, s->xo[s->read], vb, cudaMemcpyDeviceToHost));
    if (n) RT(cudaMemcpy(n, s->cf, vb, cudaMemcpyDeviceToHost));
    return 0;
}

int ref_sim_set_state(void* h, const float* x, const float* xo, const float* n) {
    auto* s = (RefSim*)h;
    size_t vb = sizeof(RVec3) * s->N;
    if (x) RT(cudaMemcpy(s->x[s->read], x, vb, cudaMemcpyHostToDevice));
    if (xo) RT(cudaMemcpy(s->xo[s->read], xo, vb, cudaMemcpyHostToDevice));
    if (n) RT(cudaMemcpy(s->cf, n, vb, cudaMemcpyHostToDevice));
    return 0;
}

int ref_sim_n_leaves(void* h) { return ((RefSim*)h)->bvh.Tp; }

// Refit race: repair = 1 makes every later build replace the internal boxes its
// unfenced refit got wrong by the ones its definition gives; the count of wrong
// boxes found in all builds so far is returned either way.
long long ref_sim_refit_race(void* h, int repair) {
    auto* s = (RefSim*)h;
    if (repair >= 0) s->bvh.repair = repair != 0;
    return (long long)s->bvh.stale;
}

// LBVH in the layout of visg_export_lbvh (link fields as BRTreeNode encodes them)
int ref_sim_export_lbvh(void* h, uint32_t* tri_codes, float* tri_boxes, uint32_t* sorted_codes, int32_t* sorted_tris,
                        int32_t* child_a, int32_t* child_b, int32_t* parent_int, int32_t* parent_leaf,
                        float* int_boxes, float* leaf_boxes, float* root_box) {
    auto* s = (RefSim*)h;
    RefBvh& b = s->bvh;
    auto put = [](float* d, const RBBox& x) {
        d[0] = x.min.x; d[1] = x.min.y; d[2] = x.min.z; d[3] = x.max.x; d[4] = x.max.y; d[5] = x.max.z;
    };
    for (int t = 0; t < b.T; ++t) {
        if (tri_codes) tri_codes[t] = b.codes[t];
        if (tri_boxes) put(tri_boxes + 6 * t, b.boxes[t]);
    }
    if (root_box) put(root_box, b.root);
    std::vector<RNode> leaf(b.Tp), in(b.Tp - 1);
    RT(cudaMemcpy(leaf.data(), b.d_leaf, sizeof(RNode) * b.Tp, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(in.data(), b.d_int, sizeof(RNode) * (b.Tp - 1), cudaMemcpyDeviceToHost));
    for (int i = 0; i < b.Tp; ++i) {
        if (sorted_codes) sorted_codes[i] = b.sorted_codes[i];
        if (sorted_tris) sorted_tris[i] = b.sorted_tris[i];
        if (parent_leaf) parent_leaf[i] = leaf[i].parent;
        if (leaf_boxes) put(leaf_boxes + 6 * i, leaf[i].bbox);
    }
    for (int i = 0; i + 1 < b.Tp; ++i) {
        if (child_a) child_a[i] = in[i].childA;
        if (child_b) child_b[i] = in[i].childB;
        if (parent_int) parent_int[i] = in[i].parent;
        if (int_boxes) put(int_boxes + 6 * i, in[i].bbox);
    }
    return 0;
}

}  // extern "C"
