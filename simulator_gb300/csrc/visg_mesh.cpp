// visg_mesh.cpp — real-mesh inputs, host only (no CUDA).
//
// visg_obj_load reads a Wavefront OBJ the way the reference's ObjLoader and
// Mesh::unified do (src/ObjLoader.cpp:14-137, src/Mesh.cpp:17-38), minus texture and
// material handling:
//   "v x y z"   a vertex (a 4th coordinate is ignored; missing ones read as 0)
//   "vn x y z"  a normal
//   "f a b c"   a triangle, 1-based vertex indices; the corner's normal index is its
//               vertex index
//   "f a/t/n b/t/n c/t/n"  the same with texture and normal indices; "a/t" takes
//               the vertex index as normal index, as the reference's parser does
//   only the first three corners of a face are kept (the reference reads three)
// Each vertex's normal is the normal named by the last face corner that uses the
// vertex (Mesh::unified assigns per corner in face order); a vertex no face uses
// keeps (0, 0, 0).  Numbers are read with strtod and rounded to float, as atof
// into glm's float vectors.
//
// visg_mesh_scale / translate / rotate are Mesh::scale, translate and rotation
// (src/Mesh.cpp:41-99), which the reference's demo applies to its garment and body
// (src/main.cpp:24-32): the centre is the float running sum of the vertices divided
// by their count (Mesh::get_center), the rotation angle is angle / 180 * 3.1415 (the
// product in double, as the literal makes it) and the rotation is the column-major
// matrix of Mesh::rotation applied to (v - centre, 1) with GLM's grouping of the
// matrix-vector sum, (c0 x + c1 y) + (c2 z + c3 w), then the centre is added back.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/visg_sim.h"

struct VisgObj {
    std::vector<float> xyz, normals;  // per vertex
    std::vector<uint32_t> faces;      // 3 per triangle
    std::vector<int32_t> groups;      // vertex counts of the "# object" records
};

namespace visg {
void set_last_error(const char* msg);  // visg_api.cu: the message of visg_last_error
}

namespace {

int obj_fail(int code, const std::string& m) {
    visg::set_last_error(m.c_str());
    return code;
}

// the index fields of one face corner: vertex, normal (0-based; -1 if unreadable)
void corner(const std::string& tok, long& v, long& n) {
    const size_t s1 = tok.find('/');
    if (s1 == std::string::npos) {
        v = std::atol(tok.c_str()) - 1;
        n = v;
        return;
    }
    v = std::atol(tok.substr(0, s1).c_str()) - 1;
    const size_t s2 = tok.find('/', s1 + 1);
    n = (s2 == std::string::npos) ? v : std::atol(tok.c_str() + s2 + 1) - 1;
}

float num(const std::string& s) { return s.empty() ? 0.0f : (float)std::strtod(s.c_str(), nullptr); }

void centre(const float* xyz, int32_t n, float c[3]) {  // Mesh::get_center
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    for (int32_t i = 0; i < n; ++i) {
        sx += xyz[3 * i];
        sy += xyz[3 * i + 1];
        sz += xyz[3 * i + 2];
    }
    c[0] = sx / (float)n;
    c[1] = sy / (float)n;
    c[2] = sz / (float)n;
}

// Nearest-neighbour search with the rules of the kd-tree library the reference
// bundles (src/kdtree.cpp: kd_insert, kd_nearest), so that ties resolve the same way:
// points are inserted in order, each node splitting on axis depth % 3 (left iff the
// point's coordinate is below the node's); the search starts from the root as its
// first guess, descends the nearer side first (left iff pos - node <= 0), then tests
// the node (a strictly smaller squared distance replaces the best), then visits the
// farther side if the bounding box of that side, clipped from the tree's box of all
// points, is strictly closer than the best.  Coordinates and distances in double.
struct KdTree {
    struct Node {
        double p[3];
        int dir, left = -1, right = -1;
        uint32_t item;
    };
    std::vector<Node> nodes;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};

    void insert(const float* xyz, uint32_t item) {
        Node nd;
        for (int k = 0; k < 3; ++k) nd.p[k] = (double)xyz[k];
        nd.item = item;
        if (nodes.empty()) {
            nd.dir = 0;
            for (int k = 0; k < 3; ++k) lo[k] = hi[k] = nd.p[k];
            nodes.push_back(nd);
            return;
        }
        for (int k = 0; k < 3; ++k) {
            if (nd.p[k] < lo[k]) lo[k] = nd.p[k];
            if (nd.p[k] > hi[k]) hi[k] = nd.p[k];
        }
        int cur = 0;
        while (true) {
            Node& c = nodes[cur];
            int& next = nd.p[c.dir] < c.p[c.dir] ? c.left : c.right;
            if (next < 0) {
                nd.dir = (c.dir + 1) % 3;
                next = (int)nodes.size();
                nodes.push_back(nd);
                return;
            }
            cur = next;
        }
    }

    static double dist_sq(const double* a, const double* b) {
        double s = 0;
        for (int k = 0; k < 3; ++k) s += (a[k] - b[k]) * (a[k] - b[k]);
        return s;
    }

    double box_dist_sq(const double* q, const double* bl, const double* bh) const {
        double s = 0;
        for (int k = 0; k < 3; ++k) {
            if (q[k] < bl[k]) s += (bl[k] - q[k]) * (bl[k] - q[k]);
            else if (q[k] > bh[k]) s += (bh[k] - q[k]) * (bh[k] - q[k]);
        }
        return s;
    }

    void search(int ni, const double* q, double* bl, double* bh, int& best, double& bd) const {
        const Node& nd = nodes[ni];
        const int dir = nd.dir;
        const bool go_left = q[dir] - nd.p[dir] <= 0;
        const int nearer = go_left ? nd.left : nd.right, farther = go_left ? nd.right : nd.left;
        double* near_c = go_left ? &bh[dir] : &bl[dir];
        double* far_c = go_left ? &bl[dir] : &bh[dir];
        if (nearer >= 0) {
            const double keep = *near_c;
            *near_c = nd.p[dir];
            search(nearer, q, bl, bh, best, bd);
            *near_c = keep;
        }
        const double d = dist_sq(nd.p, q);
        if (d < bd) {
            best = ni;
            bd = d;
        }
        if (farther >= 0) {
            const double keep = *far_c;
            *far_c = nd.p[dir];
            if (box_dist_sq(q, bl, bh) < bd) search(farther, q, bl, bh, best, bd);
            *far_c = keep;
        }
    }

    uint32_t nearest(const float* xyz) const {
        const double q[3] = {(double)xyz[0], (double)xyz[1], (double)xyz[2]};
        double bl[3] = {lo[0], lo[1], lo[2]}, bh[3] = {hi[0], hi[1], hi[2]};
        int best = 0;
        double bd = dist_sq(nodes[0].p, q);
        search(0, q, bl, bh, best, bd);
        return nodes[best].item;
    }
};

// glm::distance of two positions (vec4 with w = 1: the w term adds +0)
float fdist(const float* a, const float* b) {
    const float dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    return std::sqrt((dx * dx + dy * dy) + dz * dz);
}

}  // namespace

namespace visg {

// The reference's seams of a multi-piece garment (Springs::get_cloth_boundary_spring
// and get_boundary_boundary_spring, src/spring.cpp:98-209; SINGLE_LAYER_BOUNDARY).
// The vertices come in groups: piece 0, its boundary, piece 1, its boundary, ...
// (`sizes`, the OBJ's "# object" / "# N vertices" records).  Returns the structure
// springs create_neigh appends (spring.cpp:317-328): for every boundary vertex b and
// its nearest vertex c of its own piece, b -> c and c -> b, in boundary order; then,
// in ascending (c1, c2) order, c1 -> c2 for every pair of pieces' vertices whose
// boundary vertices are nearest neighbours across two boundaries at a distance in
// (0, 50 d), d the mean length of the first 100 boundary-to-piece pairs (of all of
// them when there are fewer: the reference reads past its array then).
int sewing_pairs(const float* xyz, int64_t n, const int32_t* sizes, int32_t n_groups,
                 std::vector<std::pair<uint32_t, uint32_t>>& out, std::string& err) {
    if (n_groups <= 0 || n_groups % 2) {
        err = "sewing needs an even number of vertex groups (piece, boundary, ...)";
        return -1;
    }
    int64_t total = 0;
    for (int32_t g = 0; g < n_groups; ++g) {
        if (sizes[g] < 0) {
            err = "negative group size";
            return -1;
        }
        total += sizes[g];
    }
    if (total > n) {
        err = "vertex groups cover more vertices than the mesh has";
        return -1;
    }
    std::vector<std::pair<uint32_t, uint32_t>> cb;  // (boundary vertex, piece vertex)
    std::vector<std::pair<int64_t, int64_t>> bspan;  // each boundary group's vertices
    int64_t s = 0;
    for (int32_t g = 0; g < n_groups; g += 2) {
        KdTree kd;
        for (int64_t i = 0; i < sizes[g]; ++i) kd.insert(xyz + 3 * (s + i), (uint32_t)(s + i));
        s += sizes[g];
        if (sizes[g] == 0 && sizes[g + 1] > 0) {
            err = "a boundary group follows an empty piece";
            return -1;
        }
        for (int64_t i = 0; i < sizes[g + 1]; ++i) cb.push_back({(uint32_t)(s + i), kd.nearest(xyz + 3 * (s + i))});
        bspan.push_back({s, s + sizes[g + 1]});
        s += sizes[g + 1];
    }
    out.clear();
    if (cb.empty()) return 0;
    const size_t navg = std::min<size_t>(100, cb.size());
    float max_dist = 0.0f;
    for (size_t i = 0; i < navg; ++i) max_dist += fdist(xyz + 3 * (size_t)cb[i].first, xyz + 3 * (size_t)cb[i].second);
    max_dist /= (float)navg;
    std::vector<std::pair<uint32_t, uint32_t>> bb;
    for (size_t i = 0; i < bspan.size(); ++i) {
        KdTree kd;
        for (size_t j = 0; j < bspan.size(); ++j)
            if (j != i)
                for (int64_t k = bspan[j].first; k < bspan[j].second; ++k) kd.insert(xyz + 3 * k, (uint32_t)k);
        if (kd.nodes.empty()) continue;
        for (int64_t k = bspan[i].first; k < bspan[i].second; ++k) {
            const uint32_t r = kd.nearest(xyz + 3 * k);
            const float d = fdist(xyz + 3 * k, xyz + 3 * (size_t)r);
            if (d < max_dist * 50.0f && d > 0.0f) bb.push_back({(uint32_t)k, r});
        }
    }
    std::vector<int64_t> piece_of(n, -1);  // boundary vertex -> its piece vertex
    for (auto& pr : cb) piece_of[pr.first] = pr.second;
    std::vector<std::pair<uint32_t, uint32_t>> seam;
    for (auto& pr : bb) seam.push_back({(uint32_t)piece_of[pr.first], (uint32_t)piece_of[pr.second]});
    std::sort(seam.begin(), seam.end());
    seam.erase(std::unique(seam.begin(), seam.end()), seam.end());
    for (auto& pr : cb) {
        out.push_back({pr.first, pr.second});
        out.push_back({pr.second, pr.first});
    }
    for (auto& pr : seam) out.push_back(pr);
    return 0;
}

}  // namespace visg

extern "C" {

int visg_obj_load(const char* path, VisgObj** out, int32_t* n_vertices, int32_t* n_faces) {
    if (!path || !out) return obj_fail(VISG_ERR_INVALID_ARG, "path or out is NULL");
    *out = nullptr;
    std::ifstream in(path);
    if (!in) return obj_fail(VISG_ERR_INVALID_ARG, std::string("cannot open ") + path);
    auto* o = new VisgObj();
    std::vector<float> vn;
    std::vector<long> corners;  // vertex, normal per corner
    std::string line;
    while (std::getline(in, line)) {
        std::stringstream ss(line);
        std::string f0, f1, f2, f3;
        ss >> f0 >> f1 >> f2 >> f3;
        if (f0 == "mtllib") {
        } else if (f1 == "object") {  // "# object NAME": a vertex group (ObjLoader.cpp:33-36)
            o->groups.push_back(0);
        } else if (f2 == "vertices") {  // "# N vertices": its size (ObjLoader.cpp:37-40)
            if (!o->groups.empty()) o->groups.back() = (int32_t)std::atol(f1.c_str());
        } else if (f0 == "v") {
            o->xyz.push_back(num(f1));
            o->xyz.push_back(num(f2));
            o->xyz.push_back(num(f3));
        } else if (f0 == "vn") {
            vn.push_back(num(f1));
            vn.push_back(num(f2));
            vn.push_back(num(f3));
        } else if (f0 == "f") {
            long v, n;
            for (const std::string* t : {&f1, &f2, &f3}) {
                corner(*t, v, n);
                corners.push_back(v);
                corners.push_back(n);
            }
        }
    }
    const long nv = (long)o->xyz.size() / 3, nn = (long)vn.size() / 3;
    o->normals.assign(o->xyz.size(), 0.0f);
    for (size_t k = 0; k < corners.size(); k += 2) {
        const long v = corners[k], n = corners[k + 1];
        if (v < 0 || v >= nv) {
            delete o;
            return obj_fail(VISG_ERR_INVALID_ARG, std::string(path) + ": face vertex index out of range");
        }
        o->faces.push_back((uint32_t)v);
        if (n >= 0 && n < nn)
            for (int j = 0; j < 3; ++j) o->normals[3 * v + j] = vn[3 * n + j];
    }
    if (nv > 0x7fffffffL || (long)o->faces.size() / 3 > 0x7fffffffL) {
        delete o;
        return obj_fail(VISG_ERR_INVALID_ARG, std::string(path) + ": too large");
    }
    *out = o;
    if (n_vertices) *n_vertices = (int32_t)nv;
    if (n_faces) *n_faces = (int32_t)(o->faces.size() / 3);
    return VISG_OK;
}

int visg_obj_get(const VisgObj* o, float* xyz, float* normals, uint32_t* faces) {
    if (!o) return obj_fail(VISG_ERR_INVALID_ARG, "obj is NULL");
    if (xyz && !o->xyz.empty()) std::memcpy(xyz, o->xyz.data(), o->xyz.size() * 4);
    if (normals && !o->normals.empty()) std::memcpy(normals, o->normals.data(), o->normals.size() * 4);
    if (faces && !o->faces.empty()) std::memcpy(faces, o->faces.data(), o->faces.size() * 4);
    return VISG_OK;
}

int visg_obj_groups(const VisgObj* o, int32_t* sizes, int32_t* n_groups) {
    if (!o) return obj_fail(VISG_ERR_INVALID_ARG, "obj is NULL");
    if (n_groups) *n_groups = (int32_t)o->groups.size();
    if (sizes && !o->groups.empty()) std::memcpy(sizes, o->groups.data(), o->groups.size() * 4);
    return VISG_OK;
}

void visg_obj_free(VisgObj* o) { delete o; }

int visg_mesh_scale(float* xyz, int32_t n, float s) {
    if (!xyz || n <= 0) return obj_fail(VISG_ERR_INVALID_ARG, "xyz is NULL or n <= 0");
    float c[3];
    centre(xyz, n, c);
    for (int32_t i = 0; i < n; ++i)
        for (int j = 0; j < 3; ++j) xyz[3 * i + j] = (xyz[3 * i + j] - c[j]) * s;
    return VISG_OK;
}

int visg_mesh_translate(float* xyz, int32_t n, float dx, float dy, float dz) {
    if (!xyz || n < 0) return obj_fail(VISG_ERR_INVALID_ARG, "xyz is NULL or n < 0");
    for (int32_t i = 0; i < n; ++i) {
        xyz[3 * i] += dx;
        xyz[3 * i + 1] += dy;
        xyz[3 * i + 2] += dz;
    }
    return VISG_OK;
}

int visg_mesh_rotate(float* xyz, int32_t n, float angle_degrees, int32_t axis) {
    if (!xyz || n <= 0) return obj_fail(VISG_ERR_INVALID_ARG, "xyz is NULL or n <= 0");
    if (axis < 0 || axis > 2) return obj_fail(VISG_ERR_INVALID_ARG, "axis must be 0 (x), 1 (y) or 2 (z)");
    const float a = (float)((double)(angle_degrees / 180.0f) * 3.1415);
    const float cs = std::cos(a), sn = std::sin(a);
    // columns c0..c3 of Mesh::rotation's matrix (its initialiser lists are columns)
    float m[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    if (axis == 0) {
        m[1][1] = cs; m[1][2] = -sn; m[2][1] = sn; m[2][2] = cs;
    } else if (axis == 1) {
        m[0][0] = cs; m[0][2] = -sn; m[2][0] = sn; m[2][2] = cs;
    } else {
        m[0][0] = cs; m[0][1] = -sn; m[1][0] = sn; m[1][1] = cs;
    }
    float c[3];
    centre(xyz, n, c);
    for (int32_t i = 0; i < n; ++i) {
        const float v[4] = {xyz[3 * i] - c[0], xyz[3 * i + 1] - c[1], xyz[3 * i + 2] - c[2], 1.0f};
        for (int j = 0; j < 3; ++j) {
            const float a01 = m[0][j] * v[0] + m[1][j] * v[1];
            const float a23 = m[2][j] * v[2] + m[3][j] * v[3];
            xyz[3 * i + j] = (a01 + a23) + c[j];
        }
    }
    return VISG_OK;
}

}  // extern "C"
