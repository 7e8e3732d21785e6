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

}  // namespace

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
        if (f0 == "v") {
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
    if (xyz) std::memcpy(xyz, o->xyz.data(), o->xyz.size() * 4);
    if (normals) std::memcpy(normals, o->normals.data(), o->normals.size() * 4);
    if (faces) std::memcpy(faces, o->faces.data(), o->faces.size() * 4);
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
