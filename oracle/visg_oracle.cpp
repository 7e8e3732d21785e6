// visg_oracle.cpp — CPU restatement of the VISGSim per-step cloth pipeline.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the smoke
// check and the CPU-baseline leg of bench.py call it; the shipped library never
// links, loads or falls back to it.
//
// It restates, function by function, the reference's hot path (paths relative to
// the reference project):
//   glm semantics           dot/cross/length/normalize as GLM 0.9.9.8 documents them
//   BBox                    src/bvh/bbox.h:17-127 (identity box min=+100, max=-100)
//   expanded triangle box   src/bvh/primitive.cu:79-91, normal :136-142
//   point/plane test        src/bvh/primitive.cu:110-125 (inside iff dist <= 0)
//   Morton code             src/bvh/bvh.cu:20-41,71-79
//   sort + de-duplication   src/Utilities.h:23-67 (called at bvh.cu:283-290)
//   radix tree              src/bvh/cudaBRT.cu:9-161 (Karras 2012)
//   refit                   src/bvh/cudaBRT.cu:166-206
//   first-hit traversal     src/bvh/cudaBRT.cu:239-349
//   fused step              src/verlet.cu:24-88,129-161
//   spring topology         src/spring.cpp:30-79,286-353,374-391
//
// Every function is a template on the scalar type T of the cloth dynamics:
// T = float reproduces the reference's single-precision arithmetic operation by
// operation (build with -ffp-contract=off, no fast-math), T = double is the FP64
// oracle.  The LBVH is always float, as in the reference.
//
// Reference-compatible definitions where the reference is undefined (the same
// choices as the CUDA library, so results are comparable):
//   * root box = exact union of every expanded triangle box merged into the
//     identity box; the reference's get_bb (bvh.cu:44-69, <<<1,129>>> over 128
//     strides) skips the last T%128-1 triangles and reads past the array when
//     T%128 == 0.
//   * sort ties are broken by triangle index (stable sort); std::sort at
//     Utilities.h:30 leaves their order unspecified, which decides the triangle
//     kept by the de-duplication.
//   * T' == 1 (one distinct code): the single leaf's box is tested directly; the
//     reference would read an empty internal-node array.  T == 0: no collision.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <unordered_map>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/visg_sim.h"

namespace {

template <typename T>
struct V3 {
    T x, y, z;
};
template <typename T> inline V3<T> mk(T a, T b, T c) { return V3<T>{a, b, c}; }
template <typename T> inline V3<T> operator+(V3<T> a, V3<T> b) { return mk<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> inline V3<T> operator-(V3<T> a, V3<T> b) { return mk<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> inline V3<T> operator*(V3<T> a, T s) { return mk<T>(a.x * s, a.y * s, a.z * s); }
template <typename T> inline V3<T> operator*(T s, V3<T> a) { return mk<T>(s * a.x, s * a.y, s * a.z); }
template <typename T> inline V3<T> operator/(V3<T> a, T s) { return mk<T>(a.x / s, a.y / s, a.z / s); }
template <typename T> inline V3<T> operator/(V3<T> a, V3<T> b) { return mk<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <typename T> inline T dot(V3<T> a, V3<T> b) {
    T px = a.x * b.x, py = a.y * b.y, pz = a.z * b.z;
    return (px + py) + pz;
}
template <typename T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return mk<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename T> inline T length(V3<T> v) { return std::sqrt(dot(v, v)); }
template <typename T> inline V3<T> normalize(V3<T> v) { return v * (T(1) / std::sqrt(dot(v, v))); }
template <typename T> inline V3<T> cvt(const float* p) { return mk<T>((T)p[0], (T)p[1], (T)p[2]); }

// ---- BBox (bbox.h) -------------------------------------------------------------
struct Box {
    float mn[3], mx[3];
};
inline Box identity_box() {  // bbox.h:17-22
    Box b;
    for (int k = 0; k < 3; ++k) { b.mn[k] = 100.0f; b.mx[k] = -100.0f; }
    return b;
}
inline Box point_box(V3<float> p) {  // bbox.h:28
    Box b;
    b.mn[0] = b.mx[0] = p.x; b.mn[1] = b.mx[1] = p.y; b.mn[2] = b.mx[2] = p.z;
    return b;
}
inline void expand(Box& a, const Box& b) {  // bbox.h:62-73 (fmin/fmax)
    for (int k = 0; k < 3; ++k) {
        a.mn[k] = std::fmin(a.mn[k], b.mn[k]);
        a.mx[k] = std::fmax(a.mx[k], b.mx[k]);
    }
}
inline void expand(Box& a, V3<float> p) { expand(a, point_box(p)); }
template <typename T> inline bool box_contains(const Box& b, V3<T> p) {  // bbox.h:84-90
    return (p.x >= (T)b.mn[0] && p.x <= (T)b.mx[0]) && (p.y >= (T)b.mn[1] && p.y <= (T)b.mx[1]) &&
           (p.z >= (T)b.mn[2] && p.z <= (T)b.mx[2]);
}

// ---- triangle primitive (primitive.cu) -------------------------------------------
inline V3<float> tri_normal(V3<float> v0, V3<float> v1, V3<float> v2) {  // primitive.cu:136-142
    return normalize(cross(v1 - v0, v2 - v0));
}
inline Box expanded_box(V3<float> v0, V3<float> v1, V3<float> v2, float depth) {  // primitive.cu:79-91
    Box b = point_box(v0);
    expand(b, v1);
    expand(b, v2);
    V3<float> n = tri_normal(v0, v1, v2);
    expand(b, v0 - depth * n);
    expand(b, v1 - depth * n);
    expand(b, v2 - depth * n);
    return b;
}

// ---- Morton code (bvh.cu:20-41) ----------------------------------------------------
inline uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
inline uint32_t morton3d(V3<float> p) {
    float x = std::fmin(std::fmax(p.x * 1024.0f, 0.0f), 1023.0f);
    float y = std::fmin(std::fmax(p.y * 1024.0f, 0.0f), 1023.0f);
    float z = std::fmin(std::fmax(p.z * 1024.0f, 0.0f), 1023.0f);
    return expand_bits((uint32_t)x) * 4 + expand_bits((uint32_t)y) * 2 + expand_bits((uint32_t)z);
}
inline V3<float> centroid(const Box& b) {  // bbox.h:97-102
    V3<float> s = mk<float>(b.mn[0] + b.mx[0], b.mn[1] + b.mx[1], b.mn[2] + b.mx[2]);
    return s / 2.0f;
}
inline V3<float> unitcube_pos(const Box& root, V3<float> p) {  // bbox.h:114-127
    V3<float> mn = mk<float>(root.mn[0], root.mn[1], root.mn[2]);
    V3<float> ext = mk<float>(root.mx[0] - root.mn[0], root.mx[1] - root.mn[1], root.mx[2] - root.mn[2]);
    V3<float> o2pos = p - mn;
    if (length(ext) != 0.0f) return o2pos / ext;
    return mk<float>(0.0f, 0.0f, 0.0f);
}

inline int clz32(uint32_t v) {
    if (v == 0) return 32;
    return __builtin_clz(v);
}

// ---- LBVH -------------------------------------------------------------------------
struct Lbvh {
    int T = 0;   // triangles
    int Tp = 0;  // leaves after de-duplication (T')
    std::vector<V3<float>> verts;
    std::vector<uint32_t> tris;
    std::vector<Box> tri_box;
    std::vector<uint32_t> tri_code;
    Box root;  // Morton frame
    std::vector<uint32_t> sorted_code;
    std::vector<int32_t> sorted_tri;
    // reference BRTreeNode link fields (cudaBRT.h:34-115)
    std::vector<int32_t> childA, childB, parent_int, parent_leaf;
    std::vector<Box> int_box, leaf_box;
    // per-leaf primitive (sorted order)
    std::vector<V3<float>> leaf_v0;
    std::vector<V3<float>> leaf_n;
};

// delta / determineRange / findSplit (cudaBRT.cu:9-110)
inline int delta(int i, int j, const uint32_t* c, int n) {
    if (j < 0 || j >= n) return -1;
    return clz32(c[i] ^ c[j]);
}
inline std::pair<int, int> determine_range(const uint32_t* c, int n_internal, int i) {
    int size = n_internal + 1;
    int d = delta(i, i + 1, c, size) - delta(i, i - 1, c, size);
    d = d > 0 ? 1 : -1;
    int delta_min = delta(i, i - d, c, size);
    int lmax = 2;
    while (delta(i, i + lmax * d, c, size) > delta_min) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(i, i + (l + t) * d, c, size) > delta_min) l += t;
    int j = i + l * d;
    return i <= j ? std::make_pair(i, j) : std::make_pair(j, i);
}
inline bool is_diff_at_bit(uint32_t a, uint32_t b, int n) { return (a >> (31 - n)) != (b >> (31 - n)); }
inline int find_split(const uint32_t* c, int first, int last) {
    if (first == last) return -1;
    int cp = clz32(c[first] ^ c[last]);
    if (cp == 32) return (first + last) / 2;
    int split = first, step = last - first;
    do {
        step = (step + 1) >> 1;
        int ns = split + step;
        if (ns < last && !is_diff_at_bit(c[first], c[ns], cp)) split = ns;
    } while (step > 1);
    return split;
}

// calculateBoudingBox's result for the subtree under internal node i: every
// internal box is the identity box expanded by child A's box, then child B's,
// children before parents.  The top levels' subtrees run as parallel tasks (they
// share no node); below, one iterative post-order walk per subtree.
void refit_subtree(Lbvh& b, int i, int level) {
    auto child_box = [&](int c) -> const Box& { return c < 0 ? b.leaf_box[-c - 1] : b.int_box[c - 1]; };
    if (level < 10) {
        Lbvh* pb = &b;  // a task would copy a reference parameter's object
        for (int c : {b.childA[i], b.childB[i]}) {
            if (c > 0) {
#pragma omp task firstprivate(c, pb, level)
                refit_subtree(*pb, c - 1, level + 1);
            }
        }
#pragma omp taskwait
        Box bx = identity_box();
        expand(bx, child_box(b.childA[i]));
        expand(bx, child_box(b.childB[i]));
        b.int_box[i] = bx;
        return;
    }
    std::vector<std::pair<int, char>> stack;  // {node, children pushed}
    stack.push_back({i, 0});
    while (!stack.empty()) {
        auto& top = stack.back();
        const int k = top.first;
        if (!top.second) {
            top.second = 1;
            const int ca = b.childA[k], cb = b.childB[k];
            if (cb > 0) stack.push_back({cb - 1, 0});
            if (ca > 0) stack.push_back({ca - 1, 0});
            continue;
        }
        stack.pop_back();
        Box bx = identity_box();
        expand(bx, child_box(b.childA[k]));
        expand(bx, child_box(b.childB[k]));
        b.int_box[k] = bx;
    }
}

void build_lbvh(Lbvh& b, const float* xyz, int nv, const uint32_t* tris, int nt, float depth) {
    b.T = nt;
    b.verts.resize(nv);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nv; ++i) b.verts[i] = cvt<float>(xyz + 3 * i);
    b.tris.assign(tris, tris + 3 * (size_t)nt);
    b.tri_box.resize(nt);
    b.tri_code.resize(nt);
    if (nt == 0) { b.Tp = 0; return; }
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t)
        b.tri_box[t] = expanded_box(b.verts[tris[3 * t]], b.verts[tris[3 * t + 1]], b.verts[tris[3 * t + 2]], depth);
    // root box: identity U every box (fmin/fmax are exact, so per-thread partial
    // unions merged afterwards give the same box as one pass in order)
    b.root = identity_box();
#pragma omp parallel
    {
        Box part = identity_box();
#pragma omp for schedule(static) nowait
        for (int t = 0; t < nt; ++t) expand(part, b.tri_box[t]);
#pragma omp critical
        expand(b.root, part);
    }
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t) b.tri_code[t] = morton3d(unitcube_pos(b.root, centroid(b.tri_box[t])));
    // indices_sort (stable: ties by triangle index) + remove_redundant + filter.
    // The stable order by code is unique; it is formed here by three stable
    // counting passes over 10-bit digits of the 30-bit codes, least significant
    // first (the same permutation std::stable_sort gives, in linear time).
    std::vector<int32_t> idx(nt), tmp(nt);
    std::iota(idx.begin(), idx.end(), 0);
    for (int shift = 0; shift < 30; shift += 10) {
        std::vector<uint32_t> count(1025, 0);
        for (int k = 0; k < nt; ++k) ++count[((b.tri_code[idx[k]] >> shift) & 1023u) + 1];
        for (int d = 0; d < 1024; ++d) count[d + 1] += count[d];
        for (int k = 0; k < nt; ++k) tmp[count[(b.tri_code[idx[k]] >> shift) & 1023u]++] = idx[k];
        idx.swap(tmp);
    }
    b.sorted_code.clear();
    b.sorted_tri.clear();
    for (int k = 0; k < nt; ++k) {
        uint32_t code = b.tri_code[idx[k]];
        if (k == 0 || code != b.sorted_code.back()) {
            b.sorted_code.push_back(code);
            b.sorted_tri.push_back(idx[k]);
        }
    }
    int n = b.Tp = (int)b.sorted_code.size();
    b.leaf_box.resize(n);
    b.leaf_v0.resize(n);
    b.leaf_n.resize(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        int t = b.sorted_tri[i];
        b.leaf_box[i] = b.tri_box[t];
        V3<float> v0 = b.verts[tris[3 * t]], v1 = b.verts[tris[3 * t + 1]], v2 = b.verts[tris[3 * t + 2]];
        b.leaf_v0[i] = v0;
        b.leaf_n[i] = tri_normal(v0, v1, v2);
    }
    int ni = n - 1;
    b.childA.assign(std::max(ni, 0), 0);
    b.childB.assign(std::max(ni, 0), 0);
    b.parent_int.assign(std::max(ni, 0), 0);
    b.parent_leaf.assign(n, 0);
    b.int_box.assign(std::max(ni, 0), identity_box());
    const uint32_t* c = b.sorted_code.data();
    // processInternalNode (cudaBRT.cu:120-161); every node has one parent, so the
    // nodes are independent
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ni; ++i) {
        auto r = determine_range(c, ni, i);
        int split = find_split(c, r.first, r.second);
        if (split == -1) continue;
        bool a_leaf = split == r.first, b_leaf = split + 1 == r.second;
        b.childA[i] = a_leaf ? -split - 1 : split + 1;
        b.childB[i] = b_leaf ? -(split + 1) - 1 : (split + 1) + 1;
        if (a_leaf) b.parent_leaf[split] = i + 1; else b.parent_int[split] = i + 1;
        if (b_leaf) b.parent_leaf[split + 1] = i + 1; else b.parent_int[split + 1] = i + 1;
    }
    // calculateBoudingBox (cudaBRT.cu:166-206): internal = identity U A U B, post-order
    if (ni > 0) {
#pragma omp parallel
#pragma omp single
        refit_subtree(b, 0, 0);
    }
}
// D_BVH::intersect (cudaBRT.cu:239-285): first overlapping leaf, children tested
// pairwise, leaves before descent, left pushed before right.
template <typename T>
int first_hit(const Lbvh& b, V3<T> p) {
    if (b.Tp == 0) return -1;
    if (b.Tp == 1) return box_contains(b.leaf_box[0], p) ? 0 : -1;
    int stack[96];
    int sp = 0;
    stack[sp++] = -1;  // NULL sentinel
    int node = 0;
    do {
        int ca = b.childA[node], cb = b.childB[node];
        const Box& ba = ca < 0 ? b.leaf_box[-ca - 1] : b.int_box[ca - 1];
        const Box& bb = cb < 0 ? b.leaf_box[-cb - 1] : b.int_box[cb - 1];
        bool ol = box_contains(ba, p), orr = box_contains(bb, p);
        if (ol && ca < 0) return -ca - 1;
        if (orr && cb < 0) return -cb - 1;
        bool tl = ol && ca > 0, tr = orr && cb > 0;
        if (!tl && !tr) node = stack[--sp];
        else {
            node = tl ? ca - 1 : cb - 1;
            if (tl && tr) stack[sp++] = cb - 1;
        }
    } while (node != -1);
    return -1;
}

// Primitive::d_intersect (primitive.cu:110-125)
template <typename T>
bool prim_intersect(const Lbvh& b, int leaf, V3<T> p, T& dist, V3<T>& normal) {
    int t = b.sorted_tri[leaf];
    V3<T> v0 = mk<T>((T)b.verts[b.tris[3 * t]].x, (T)b.verts[b.tris[3 * t]].y, (T)b.verts[b.tris[3 * t]].z);
    V3<T> v1 = mk<T>((T)b.verts[b.tris[3 * t + 1]].x, (T)b.verts[b.tris[3 * t + 1]].y, (T)b.verts[b.tris[3 * t + 1]].z);
    V3<T> v2 = mk<T>((T)b.verts[b.tris[3 * t + 2]].x, (T)b.verts[b.tris[3 * t + 2]].y, (T)b.verts[b.tris[3 * t + 2]].z);
    normal = normalize(cross(v1 - v0, v2 - v0));
    dist = dot(p - v0, normal);
    return !(dist > (T)0);
}

// ---- simulation --------------------------------------------------------------------
struct List {
    std::vector<uint32_t> row;
    std::vector<VisgSpring> ent;
    std::vector<float> k;  // empty = list constant
};

template <typename T>
struct Sim {
    VisgParams p;
    int N = 0;
    std::vector<List> lists;
    std::vector<V3<T>> x[2], xo[2], n;
    std::vector<char> pinned;
    int cur = 0;
    Lbvh bvh;
    std::vector<float> body_raw;  // as given (before thickness push)
    int nv = 0;
    // adjoint records
    int ckpt_every = 0, nsteps_fwd = 0;
    std::vector<std::vector<V3<T>>> ck_x, ck_xo, ck_n;

    void set_body(const float* xyz, const float* normals) {
        std::vector<float> v(xyz, xyz + 3 * (size_t)nv);
        if (normals) {  // Mesh::vertex_extend (Mesh.cpp:101-117): v += dist * n, once per vertex
            for (int i = 0; i < 3 * nv; ++i) v[i] = v[i] + p.thickness * normals[i];
        }
        body_raw = v;
        std::vector<uint32_t> tr = bvh.tris;
        build_lbvh(bvh, v.data(), nv, tr.data(), (int)tr.size() / 3, p.box_depth);
    }

    // collision_response_projection (verlet.cu:24-50); *leaf_used = the leaf the
    // vertex was projected onto, or -1
    bool collide(V3<T>& pos, V3<T>& pos_old, V3<T>& nrm, int* leaf_used = nullptr) const {
        int leaf = first_hit(bvh, pos);
        if (leaf_used) *leaf_used = -1;
        if (leaf >= 0) {
            T dist;
            V3<T> normal;
            if (prim_intersect(bvh, leaf, pos, dist, normal)) {
                T k = (T)1.0;
                dist = k * std::fabs(dist);
                pos = pos + dist * normal;
                pos_old = pos;
                nrm = normal;
                if (leaf_used) *leaf_used = leaf;
                return true;
            }
        }
        nrm = mk<T>(0, 0, 0);
        return false;
    }

    // Contact replay (a check of derivatives, not part of the reference's algorithm):
    // when `forced` is set, the step does not decide contacts; vertex i is projected
    // onto the plane of leaf forced[i] (or not at all for -1) by the branch's own
    // formula x' = x* - ((x* - v0) . n) n, which for dist <= 0 is the reference's
    // x* + |dist| n to the last bit.  `record`, when set, receives the leaf each
    // vertex of an ordinary step was projected onto.  A forward pass replayed with
    // another parameter value then stays on the recorded contact history, so its
    // difference quotients are derivatives of the same piece of the trajectory that
    // a frozen-active-set adjoint differentiates.
    const int* forced = nullptr;
    int* record = nullptr;

    // verlet kernel body (verlet.cu:129-161) for one vertex; writes outputs.
    void vertex_step(int i, const std::vector<V3<T>>& X, const std::vector<V3<T>>& XO,
                     V3<T>& xout, V3<T>& xoout) {
        V3<T> pos = X[i], pos_old = XO[i];
        if (pinned[i]) {
            xout = pos;
            xoout = pos;
            n[i] = mk<T>(0, 0, 0);
            if (record) record[i] = -1;
            return;
        }
        const T dt = (T)p.dt, mass = (T)p.mass, damp = (T)p.force_damping, kd = (T)p.spring_damping;
        V3<T> vel = (pos - pos_old) / dt;
        V3<T> gravity = mk<T>((T)p.gravity[0], (T)p.gravity[1], (T)p.gravity[2]);
        V3<T> force = gravity * mass + vel * damp;
        for (size_t l = 0; l < lists.size(); ++l) {  // compute_spring_force (verlet.cu:52-88)
            const List& L = lists[l];
            V3<T> f = mk<T>(0, 0, 0);
            for (uint32_t e = L.row[i]; e < L.row[i + 1]; ++e) {
                T ks = L.k.empty() ? (T)p.list_k[l] : (T)L.k[e];
                int j = L.ent[e].end;
                V3<T> p2 = X[j], p2_last = XO[j];
                V3<T> v2 = (p2 - p2_last) / dt;
                V3<T> deltaP = pos - p2;
                const T eps = (T)FLT_EPSILON_T;
                deltaP = deltaP + mk<T>(eps, eps, eps);
                V3<T> deltaV = vel - v2;
                T dist = length(deltaP);
                T original = (T)L.ent[e].rest;
                T leftTerm = -ks * (dist - original);
                T rightTerm = kd * (dot(deltaV, deltaP) / dist);
                V3<T> springForce = (leftTerm + rightTerm) * normalize(deltaP);
                f = f + springForce;
            }
            force = force + f;
        }
        V3<T> cf = n[i];
        V3<T> inelastic = dot(cf, force) * cf;
        force = force - inelastic;
        V3<T> acc = force / mass;
        V3<T> tmp = pos;
        if (p.verlet_damping == 1.0f)
            pos = ((pos + pos) - pos_old) + ((acc * dt) * dt);
        else
            pos = (pos + ((T)p.verlet_damping * (pos - pos_old))) + ((acc * dt) * dt);
        pos_old = tmp;
        if (p.collide && bvh.Tp > 0 && forced) {
            const int lf = forced[i];
            if (lf >= 0) {
                T dist;
                V3<T> normal;
                prim_intersect(bvh, lf, pos, dist, normal);
                pos = pos - dist * normal;
                pos_old = pos;
                n[i] = normal;
            } else {
                n[i] = mk<T>(0, 0, 0);
            }
        } else if (p.collide && bvh.Tp > 0) {
            V3<T> nn;
            collide(pos, pos_old, nn, record ? record + i : nullptr);
            n[i] = nn;
        } else {
            n[i] = mk<T>(0, 0, 0);
        }
        xout = pos;
        xoout = pos_old;
    }
    static constexpr double FLT_EPSILON_T = 1.1920928955078125e-07;  // FLT_EPSILON

    void step() {
        const auto& X = x[cur];
        const auto& XO = xo[cur];
        auto& Y = x[cur ^ 1];
        auto& YO = xo[cur ^ 1];
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) vertex_step(i, X, XO, Y[i], YO[i]);
        cur ^= 1;
        // the contact set of this step (which vertices were projected, along which
        // normal) folded into a running hash: two runs with equal hashes had equal
        // contact sets in every step (up to a hash collision)
        uint64_t h = contact_hash ^ (0x9e3779b97f4a7c15ull * (uint64_t)(++steps_taken));
        for (int i = 0; i < N; ++i) {
            if (n[i].x == 0 && n[i].y == 0 && n[i].z == 0) continue;
            const double c[3] = {(double)n[i].x, (double)n[i].y, (double)n[i].z};
            uint64_t w[3];
            std::memcpy(w, c, sizeof w);
            for (uint64_t v : {(uint64_t)i, w[0], w[1], w[2]}) {
                h ^= v;
                h *= 0x100000001b3ull;  // FNV-1a-style mixing over 64-bit words
                h ^= h >> 29;
            }
        }
        contact_hash = h;
    }
    uint64_t contact_hash = 0;
    uint64_t steps_taken = 0;

    // ---------------- adjoint (FP64 reference gradient) ----------------
    // One step with the contact set frozen: contact[i] >= 0 marks vertices that
    // were projected, with projection normal nu[i]; nprev = normals entering the step.
    struct StepRec {
        std::vector<V3<T>> x, xo, nprev, nu;
        std::vector<char> hit;
    };
    void record_step(StepRec& r) {
        r.x = x[cur]; r.xo = xo[cur]; r.nprev = n;
        step();
        r.nu = n;
        r.hit.resize(N);
        for (int i = 0; i < N; ++i) r.hit[i] = (n[i].x != 0 || n[i].y != 0 || n[i].z != 0);
    }
    // The reverse sweep runs in double whatever T is: with T = float it is the exact
    // derivative of the float trajectory (per-step contributions of both signs cancel
    // over many steps, which float accumulation would not resolve).
    using D = double;
    static V3<D> up(const V3<T>& v) { return mk<D>((D)v.x, (D)v.y, (D)v.z); }
    // Spring force derivative helper for entry i->j; returns the contributions of
    // adjoint G (of the force on i) to (x_i, xo_i, x_j, xo_j) and dF/dk, dF/dkd.
    void spring_adj(const V3<D>& xi, const V3<D>& xoi, const V3<D>& xj, const V3<D>& xoj, D ks, D L0,
                    const V3<D>& G, V3<D>& gxi, V3<D>& gxoi, V3<D>& gxj, V3<D>& gxoj, D& gk, D& gkd) const {
        const D dt = (D)p.dt, kd = (D)p.spring_damping;
        const D eps = (D)FLT_EPSILON_T;
        V3<D> vi = (xi - xoi) / dt, vj = (xj - xoj) / dt;
        V3<D> d = (xi - xj) + mk<D>(eps, eps, eps);
        V3<D> dv = vi - vj;
        D L = length(d);
        V3<D> u = d / L;
        D dvu = dot(dv, u);
        D s = -ks * (L - L0) + kd * dvu;
        D uG = dot(u, G);
        // ds/dd = -ks u + kd/L (dv - dvu u); d(u)/dd = (I - u u^T)/L
        V3<D> dsdd = (-ks) * u + (kd / L) * (dv - dvu * u);
        V3<D> gd = uG * dsdd + (s / L) * (G - uG * u);
        V3<D> gdv = (kd * uG) * u;
        gxi = gd + gdv / dt;
        gxoi = (D(-1) / dt) * gdv;
        gxj = mk<D>(0, 0, 0) - gxi;
        gxoj = mk<D>(0, 0, 0) - gxoi;
        gk = -(L - L0) * uG;
        gkd = dvu * uG;
    }
    // Backward through one recorded step: lx, lxo are adjoints of the step's outputs
    // on entry and of its inputs on return.
    void backward_step(const StepRec& r, std::vector<V3<D>>& lx, std::vector<V3<D>>& lxo,
                       std::vector<std::vector<double>>& dk, double& dgamma, double& dc, double& dkd) {
        const D dt = (D)p.dt, mass = (D)p.mass, gamma = (D)p.verlet_damping;
        std::vector<V3<D>> G(N), nlx(N, mk<D>(0, 0, 0)), nlxo(N, mk<D>(0, 0, 0));
        for (int i = 0; i < N; ++i) {
            if (pinned[i]) { nlx[i] = nlx[i] + lx[i] + lxo[i]; G[i] = mk<D>(0, 0, 0); continue; }
            V3<D> lstar;
            if (r.hit[i]) {
                V3<D> a = lx[i] + lxo[i];
                V3<D> nu = up(r.nu[i]);
                lstar = a - dot(nu, a) * nu;
            } else {
                lstar = lx[i];
                nlx[i] = nlx[i] + lxo[i];
            }
            const V3<D> xi = up(r.x[i]), xoi = up(r.xo[i]);
            nlx[i] = nlx[i] + (D(1) + gamma) * lstar;
            nlxo[i] = nlxo[i] - gamma * lstar;
            dgamma += dot(lstar, xi - xoi);
            V3<D> h = ((dt * dt) / mass) * lstar;
            V3<D> np = up(r.nprev[i]);
            G[i] = h - dot(np, h) * np;
            V3<D> v = (xi - xoi) / dt;
            dc += dot(G[i], v);
            D c = (D)p.force_damping;
            nlx[i] = nlx[i] + (c / dt) * G[i];
            nlxo[i] = nlxo[i] - (c / dt) * G[i];
        }
        for (int i = 0; i < N; ++i) {
            if (pinned[i]) continue;
            for (size_t l = 0; l < lists.size(); ++l) {
                const List& Ls = lists[l];
                for (uint32_t e = Ls.row[i]; e < Ls.row[i + 1]; ++e) {
                    D ks = Ls.k.empty() ? (D)p.list_k[l] : (D)Ls.k[e];
                    int j = Ls.ent[e].end;
                    V3<D> gxi, gxoi, gxj, gxoj;
                    D gk, gkd;
                    spring_adj(up(r.x[i]), up(r.xo[i]), up(r.x[j]), up(r.xo[j]), ks, (D)Ls.ent[e].rest, G[i], gxi, gxoi,
                               gxj, gxoj, gk, gkd);
                    nlx[i] = nlx[i] + gxi;
                    nlxo[i] = nlxo[i] + gxoi;
                    nlx[j] = nlx[j] + gxj;
                    nlxo[j] = nlxo[j] + gxoj;
                    dk[l][e] += gk;
                    dkd += gkd;
                }
            }
        }
        lx.swap(nlx);
        lxo.swap(nlxo);
    }
};

template <typename T>
Sim<T>* make_sim(const VisgParams* p, const float* cloth, int N, const uint32_t* const* rows,
                 const VisgSpring* const* ents, const float* const* ks, const float* body, const float* bn,
                 int nv, const uint32_t* tris, int nt) {
    auto* s = new Sim<T>();
    s->p = *p;
    s->N = N;
    s->lists.resize(p->n_lists);
    for (int l = 0; l < p->n_lists; ++l) {
        s->lists[l].row.assign(rows[l], rows[l] + N + 1);
        uint32_t E = rows[l][N];
        s->lists[l].ent.assign(ents[l], ents[l] + E);
        if (ks && ks[l]) s->lists[l].k.assign(ks[l], ks[l] + E);
    }
    for (int b = 0; b < 2; ++b) { s->x[b].resize(N); s->xo[b].resize(N); }
    s->n.assign(N, mk<T>(0, 0, 0));
    s->pinned.assign(N, 0);
    for (int i = 0; i < N; ++i) s->x[0][i] = s->xo[0][i] = cvt<T>(cloth + 3 * i);
    s->nv = nv;
    s->bvh.tris.assign(tris, tris + 3 * (size_t)nt);
    if (nv > 0) s->set_body(body, bn); else s->bvh.T = s->bvh.Tp = 0;
    return s;
}

struct Handle {
    int prec;  // 4 or 8
    void* sim;
};

}  // namespace

// =====================================================================================
// C entry points (ctypes)
// =====================================================================================
extern "C" {

int orc_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

void* orc_sim_create(int prec, const VisgParams* p, const float* cloth, int N, const uint32_t* const* rows,
                     const VisgSpring* const* ents, const float* const* ks, const float* body, const float* bn,
                     int nv, const uint32_t* tris, int nt) {
    auto* h = new Handle();
    h->prec = prec;
    if (prec == 8) h->sim = make_sim<double>(p, cloth, N, rows, ents, ks, body, bn, nv, tris, nt);
    else h->sim = make_sim<float>(p, cloth, N, rows, ents, ks, body, bn, nv, tris, nt);
    return h;
}

void orc_sim_destroy(void* hv) {
    auto* h = (Handle*)hv;
    if (h->prec == 8) delete (Sim<double>*)h->sim; else delete (Sim<float>*)h->sim;
    delete h;
}

#define ORC_DISPATCH(hv, ...)                                               \
    do {                                                                    \
        auto* h_ = (Handle*)(hv);                                           \
        if (h_->prec == 8) { auto* s = (Sim<double>*)h_->sim; __VA_ARGS__; } \
        else { auto* s = (Sim<float>*)h_->sim; __VA_ARGS__; }               \
    } while (0)

void orc_sim_step(void* hv, int nsteps) {
    ORC_DISPATCH(hv, for (int k = 0; k < nsteps; ++k) s->step());
}

void orc_sim_update_body(void* hv, const float* xyz, const float* normals) {
    ORC_DISPATCH(hv, s->set_body(xyz, normals));
}

void orc_sim_set_vertex(void* hv, int idx, const float* xyz) {
    ORC_DISPATCH(hv, {
        using TT = std::remove_reference_t<decltype(s->x[0][0].x)>;
        s->x[s->cur][idx] = mk<TT>((TT)xyz[0], (TT)xyz[1], (TT)xyz[2]);
        s->xo[s->cur][idx] = s->x[s->cur][idx];
    });
}

void orc_sim_set_pinned(void* hv, const uint32_t* idx, int n) {
    ORC_DISPATCH(hv, {
        std::fill(s->pinned.begin(), s->pinned.end(), 0);
        for (int k = 0; k < n; ++k) s->pinned[idx[k]] = 1;
    });
}

// state as doubles (N*3 each); any pointer may be NULL
void orc_sim_get_state(void* hv, double* x, double* xo, double* n) {
    ORC_DISPATCH(hv, {
        for (int i = 0; i < s->N; ++i) {
            auto a = s->x[s->cur][i], b = s->xo[s->cur][i], c = s->n[i];
            if (x) { x[3 * i] = a.x; x[3 * i + 1] = a.y; x[3 * i + 2] = a.z; }
            if (xo) { xo[3 * i] = b.x; xo[3 * i + 1] = b.y; xo[3 * i + 2] = b.z; }
            if (n) { n[3 * i] = c.x; n[3 * i + 1] = c.y; n[3 * i + 2] = c.z; }
        }
    });
}

void orc_sim_set_state(void* hv, const float* x, const float* xo, const float* n) {
    ORC_DISPATCH(hv, {
        using TT = std::remove_reference_t<decltype(s->x[0][0].x)>;
        for (int i = 0; i < s->N; ++i) {
            if (x) s->x[s->cur][i] = cvt<TT>(x + 3 * i);
            if (xo) s->xo[s->cur][i] = cvt<TT>(xo + 3 * i);
            if (n) s->n[i] = cvt<TT>(n + 3 * i);
        }
    });
}

// Contact record / replay (see Sim::forced): orc_sim_record_contacts steps nsteps
// times, keeping the leaf every vertex was projected onto in every step, and
// returns the record; orc_sim_step_forced replays steps [first, first + n) of a
// record (on a simulator of the same cloth and body); orc_contacts_free frees it.
struct ContactRecord {
    int n = 0;
    std::vector<std::vector<int>> leaf;  // per step, per vertex: leaf or -1
};
void* orc_sim_record_contacts(void* hv, int nsteps) {
    auto* rec = new ContactRecord();
    ORC_DISPATCH(hv, {
        rec->n = s->N;
        rec->leaf.assign(nsteps, std::vector<int>(s->N, -1));
        for (int k = 0; k < nsteps; ++k) {
            s->record = rec->leaf[k].data();
            s->step();
        }
        s->record = nullptr;
    });
    return rec;
}
int orc_sim_step_forced(void* hv, void* recv, int first, int nsteps) {
    auto* rec = (ContactRecord*)recv;
    int bad = 0;
    ORC_DISPATCH(hv, {
        if (rec->n != s->N || first < 0 || first + nsteps > (int)rec->leaf.size()) {
            bad = 1;
        } else {
            for (int k = 0; k < nsteps; ++k) {
                s->forced = rec->leaf[first + k].data();
                s->step();
            }
            s->forced = nullptr;
        }
    });
    return bad ? -1 : 0;
}
void orc_contacts_free(void* recv) { delete (ContactRecord*)recv; }

// Running hash of every step's contact set since the simulator was created.
uint64_t orc_sim_contact_hash(void* hv) {
    uint64_t r = 0;
    ORC_DISPATCH(hv, r = s->contact_hash);
    return r;
}

int orc_sim_n_leaves(void* hv) {
    int r = 0;
    ORC_DISPATCH(hv, r = s->bvh.Tp);
    return r;
}

// LBVH export in the reference layout (see visg_export_lbvh); any pointer may be NULL.
void orc_sim_export_lbvh(void* hv, uint32_t* tri_codes, float* tri_boxes, uint32_t* sorted_codes,
                         int32_t* sorted_tris, int32_t* child_a, int32_t* child_b, int32_t* parent_int,
                         int32_t* parent_leaf, float* int_boxes, float* leaf_boxes, float* root_box) {
    ORC_DISPATCH(hv, {
        const Lbvh& b = s->bvh;
        auto put = [](float* dst, const Box& bx) {
            for (int k = 0; k < 3; ++k) { dst[k] = bx.mn[k]; dst[3 + k] = bx.mx[k]; }
        };
        for (int t = 0; t < b.T; ++t) {
            if (tri_codes) tri_codes[t] = b.tri_code[t];
            if (tri_boxes) put(tri_boxes + 6 * t, b.tri_box[t]);
        }
        for (int i = 0; i < b.Tp; ++i) {
            if (sorted_codes) sorted_codes[i] = b.sorted_code[i];
            if (sorted_tris) sorted_tris[i] = b.sorted_tri[i];
            if (parent_leaf) parent_leaf[i] = b.parent_leaf[i];
            if (leaf_boxes) put(leaf_boxes + 6 * i, b.leaf_box[i]);
        }
        for (int i = 0; i + 1 < b.Tp; ++i) {
            if (child_a) child_a[i] = b.childA[i];
            if (child_b) child_b[i] = b.childB[i];
            if (parent_int) parent_int[i] = b.parent_int[i];
            if (int_boxes) put(int_boxes + 6 * i, b.int_box[i]);
        }
        if (root_box && b.T > 0) put(root_box, b.root);
    });
}

// First-hit query of the current LBVH (float points, evaluated in the handle's precision)
void orc_sim_query(void* hv, const float* pts, int n, int32_t* leaf, int32_t* inside, double* dist,
                   double* normal) {
    ORC_DISPATCH(hv, {
        using TT = std::remove_reference_t<decltype(s->x[0][0].x)>;
        for (int i = 0; i < n; ++i) {
            V3<TT> q = cvt<TT>(pts + 3 * i);
            int lf = first_hit(s->bvh, q);
            TT d = 0;
            V3<TT> nn = mk<TT>(0, 0, 0);
            int in = 0;
            if (lf >= 0) in = prim_intersect(s->bvh, lf, q, d, nn) ? 1 : 0;
            if (leaf) leaf[i] = lf;
            if (inside) inside[i] = in;
            if (dist) dist[i] = (double)d;
            if (normal) { normal[3 * i] = nn.x; normal[3 * i + 1] = nn.y; normal[3 * i + 2] = nn.z; }
        }
    });
}

// Forward for the adjoint: the state (x, x_old, normal) every `ckpt` steps and at the
// end; the backward pass replays each segment from its checkpoint (same results, so
// the same contact set) and walks it in reverse.
}  // extern "C"

template <typename T>
struct Tape {
    int nsteps = 0, ckpt = 1;
    std::vector<std::vector<V3<T>>> cx, cxo, cn;  // checkpoints
    std::vector<V3<T>> fx, fxo, fn;               // final state
};

extern "C" {

int orc_sim_forward(void* hv, int nsteps, int ckpt, void** tape_out) {
    ORC_DISPATCH(hv, {
        using TT = std::remove_reference_t<decltype(s->x[0][0].x)>;
        auto* tp = new Tape<TT>();
        tp->nsteps = nsteps;
        tp->ckpt = ckpt < 1 ? 1 : ckpt;
        for (int k = 0; k < nsteps; ++k) {
            if (k % tp->ckpt == 0) {
                tp->cx.push_back(s->x[s->cur]);
                tp->cxo.push_back(s->xo[s->cur]);
                tp->cn.push_back(s->n);
            }
            s->step();
        }
        tp->fx = s->x[s->cur];
        tp->fxo = s->xo[s->cur];
        tp->fn = s->n;
        *tape_out = tp;
    });
    return 0;
}

void orc_sim_backward(void* hv, void* tape, const double* dL_dx, const double* dL_dxo, double* dk_out,
                      double* dscalar) {
    ORC_DISPATCH(hv, {
        using TT = std::remove_reference_t<decltype(s->x[0][0].x)>;
        auto* tp = (Tape<TT>*)tape;
        std::vector<V3<double>> lx(s->N), lxo(s->N);
        for (int i = 0; i < s->N; ++i) {
            lx[i] = mk<double>(dL_dx[3 * i], dL_dx[3 * i + 1], dL_dx[3 * i + 2]);
            lxo[i] = dL_dxo ? mk<double>(dL_dxo[3 * i], dL_dxo[3 * i + 1], dL_dxo[3 * i + 2]) : mk<double>(0, 0, 0);
        }
        std::vector<std::vector<double>> dk(s->lists.size());
        for (size_t l = 0; l < s->lists.size(); ++l) dk[l].assign(s->lists[l].ent.size(), 0.0);
        double dg = 0, dc = 0, dkd = 0;
        const int nseg = (int)tp->cx.size();
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int s0 = seg * tp->ckpt, s1 = std::min(s0 + tp->ckpt, tp->nsteps);
            s->x[s->cur] = tp->cx[seg];
            s->xo[s->cur] = tp->cxo[seg];
            s->n = tp->cn[seg];
            std::vector<typename Sim<TT>::StepRec> recs(s1 - s0);
            for (int k = 0; k < s1 - s0; ++k) s->record_step(recs[k]);
            for (int k = s1 - s0 - 1; k >= 0; --k) s->backward_step(recs[k], lx, lxo, dk, dg, dc, dkd);
        }
        s->x[s->cur] = tp->fx;
        s->xo[s->cur] = tp->fxo;
        s->n = tp->fn;
        size_t off = 0;
        for (size_t l = 0; l < dk.size(); ++l)
            for (size_t e = 0; e < dk[l].size(); ++e) dk_out[off++] = dk[l][e];
        dscalar[0] = dg; dscalar[1] = dc; dscalar[2] = dkd;
        delete tp;
    });
}

// Output stage of Simulator::cuda_update_vbo (simulation.cu:196-231), headless.
//   update_vbo_pos      (verlet.cu:119-127): pos4[i] = vec4(x[i], 1)
//   compute_face_normal (verlet.cu:91-116):  fn[f] = normalize(cross(p1 - p0, p2 - p0)) of x_prev
//   get_vertex_adjface  (simulation.cu:152-180): faces of each vertex, in face order
//   compute_vbo_normal  (verlet.cu:163-181): vn[i] = normalize(sum of its faces' normals)
// x are the positions after the step (x_cur_out), x_prev the ones the step started
// from (x_cur_in: the reference computes normals from them).  Any output may be NULL.
void orc_render(const float* x, const float* x_prev, int n, const uint32_t* faces, int nf, float* pos4,
                float* vnormal, float* fnormal) {
    if (pos4)
        for (int i = 0; i < n; ++i) {
            pos4[4 * i] = x[3 * i];
            pos4[4 * i + 1] = x[3 * i + 1];
            pos4[4 * i + 2] = x[3 * i + 2];
            pos4[4 * i + 3] = 1.0f;
        }
    std::vector<V3<float>> fn(nf);
    for (int f = 0; f < nf; ++f) {
        const V3<float> p0 = cvt<float>(x_prev + 3 * (size_t)faces[3 * f]);
        const V3<float> p1 = cvt<float>(x_prev + 3 * (size_t)faces[3 * f + 1]);
        const V3<float> p2 = cvt<float>(x_prev + 3 * (size_t)faces[3 * f + 2]);
        fn[f] = normalize(cross(p1 - p0, p2 - p0));
        if (fnormal) { fnormal[3 * f] = fn[f].x; fnormal[3 * f + 1] = fn[f].y; fnormal[3 * f + 2] = fn[f].z; }
    }
    if (!vnormal) return;
    std::vector<std::vector<uint32_t>> adj(n);
    for (int f = 0; f < nf; ++f)
        for (int j = 0; j < 3; ++j) adj[faces[3 * f + j]].push_back((uint32_t)f);
    for (int i = 0; i < n; ++i) {
        V3<float> v = mk<float>(0.0f, 0.0f, 0.0f);
        for (uint32_t f : adj[i]) v = v + fn[f];
        v = normalize(v);
        vnormal[3 * i] = v.x; vnormal[3 * i + 1] = v.y; vnormal[3 * i + 2] = v.z;
    }
}

// The reference's fragment shader (src/shaders/sh.frag:13-55) at each vertex normal:
// diffuse = C1 L22 (x x - y y) + C3 L20 z z + C4 L00 - C5 L20 + 2 C1 L2m2 x y
//           + 2 C1 L21 x y + 2 C1 L2m1 y z + 2 C2 L11 x + 2 C2 L1m1 y + 2 C2 L10 z,
// term by term left to right on normalize(n); colour = ((0 + diffuse * 1) + 0) * rgb.
void orc_sh_shade(const float* normals, int n, const float* rgb, float* out) {
    const float C1 = 0.429043f, C2 = 0.511664f, C3 = 0.743125f, C4 = 0.886227f, C5 = 0.247708f;
    const V3<float> L00 = mk(0.87f, 0.87f, 0.86f), L1m1 = mk(0.17f, 0.24f, 0.31f), L10 = mk(0.03f, 0.03f, 0.03f);
    const V3<float> L11 = mk(-0.004f, -0.03f, -0.05f), L2m2 = mk(-0.12f, -0.12f, -0.11f);
    const V3<float> L2m1 = mk(0.003f, 0.003f, 0.007f), L20 = mk(-0.03f, -0.02f, -0.02f);
    const V3<float> L21 = mk(-0.08f, -0.08f, -0.09f), L22 = mk(-0.16f, -0.19f, -0.22f);
    const float c1x2 = 2.0f * C1, c2x2 = 2.0f * C2;
    for (int i = 0; i < n; ++i) {
        const V3<float> t = normalize(cvt<float>(normals + 3 * (size_t)i));
        V3<float> d = (C1 * L22) * (t.x * t.x - t.y * t.y);
        d = d + ((C3 * L20) * t.z) * t.z;
        d = d + C4 * L00;
        d = d - C5 * L20;
        d = d + ((c1x2 * L2m2) * t.x) * t.y;
        d = d + ((c1x2 * L21) * t.x) * t.y;
        d = d + ((c1x2 * L2m1) * t.y) * t.z;
        d = d + (c2x2 * L11) * t.x;
        d = d + (c2x2 * L1m1) * t.y;
        d = d + (c2x2 * L10) * t.z;
        d = d * 1.0f;
        const V3<float> r = (mk(0.0f, 0.0f, 0.0f) + d) + mk(0.0f, 0.0f, 0.0f);
        out[3 * i] = r.x * rgb[0];
        out[3 * i + 1] = r.y * rgb[1];
        out[3 * i + 2] = r.z * rgb[2];
    }
}

// Reference spring topology (Springs::create_neigh + CSR_spring).  Two passes like
// visg_springs_from_mesh: NULL arrays return the counts only.
int orc_springs_from_mesh(const float* xyz, int nv, const uint32_t* tris, int nt, uint32_t* row0,
                          VisgSpring* ent0, int32_t* n0, uint32_t* row1, VisgSpring* ent1, int32_t* n1) {
    std::vector<std::vector<uint32_t>> neigh1(nv), neigh2(nv);
    auto exist = [](const std::vector<uint32_t>& a, uint32_t v) { return std::find(a.begin(), a.end(), v) != a.end(); };
    for (int i = 0; i < nt; ++i) {  // spring.cpp:291-313
        uint32_t f[3] = {tris[3 * i], tris[3 * i + 1], tris[3 * i + 2]};
        if (!exist(neigh1[f[0]], f[1])) neigh1[f[0]].push_back(f[1]);
        if (!exist(neigh1[f[0]], f[2])) neigh1[f[0]].push_back(f[2]);
        if (!exist(neigh1[f[1]], f[0])) neigh1[f[1]].push_back(f[0]);
        if (!exist(neigh1[f[1]], f[2])) neigh1[f[1]].push_back(f[2]);
        if (!exist(neigh1[f[2]], f[0])) neigh1[f[2]].push_back(f[0]);
        if (!exist(neigh1[f[2]], f[1])) neigh1[f[2]].push_back(f[1]);
    }
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> mat;  // Matrix::Insert_Matrix (spring.cpp:30-79)
    std::vector<std::pair<uint32_t, uint32_t>> inl;
    auto ins = [&](uint32_t a, uint32_t b, uint32_t c) {
        auto it1 = mat.find({a, b});
        if (it1 != mat.end()) { inl.push_back({it1->second, c}); return; }
        auto it2 = mat.find({b, a});
        if (it2 != mat.end()) { inl.push_back({it2->second, c}); return; }
        mat.insert({{a, b}, c});
    };
    for (int i = 0; i < nt; ++i) {  // spring.cpp:331-341
        uint32_t f[3] = {tris[3 * i], tris[3 * i + 1], tris[3 * i + 2]};
        ins(f[0], f[1], f[2]);
        ins(f[0], f[2], f[1]);
        ins(f[1], f[2], f[0]);
    }
    for (auto& pr : inl) { neigh2[pr.first].push_back(pr.second); neigh2[pr.second].push_back(pr.first); }
    auto emit = [&](const std::vector<std::vector<uint32_t>>& nb, uint32_t* row, VisgSpring* ent, int32_t* cnt) {
        size_t c = 0;
        for (int i = 0; i < nv; ++i) {  // CSR_spring (spring.cpp:374-391)
            if (row) row[i] = (uint32_t)c;
            for (uint32_t j : nb[i]) {
                if (ent) {
                    float dx = xyz[3 * j] - xyz[3 * i], dy = xyz[3 * j + 1] - xyz[3 * i + 1], dz = xyz[3 * j + 2] - xyz[3 * i + 2];
                    float px = dx * dx, py = dy * dy, pz = dz * dz;
                    ent[c].end = (int32_t)j;
                    ent[c].rest = std::sqrt(((px + py) + pz) + 0.0f);
                }
                ++c;
            }
        }
        if (row) row[nv] = (uint32_t)c;
        *cnt = (int32_t)c;
    };
    emit(neigh1, row0, ent0, n0);
    emit(neigh2, row1, ent1, n1);
    return 0;
}

}  // extern "C"
