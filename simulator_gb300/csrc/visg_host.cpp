// visg_host.cpp — host-only helpers of the C ABI (no CUDA).
//
// visg_springs_from_mesh builds the reference's two spring lists from a triangle
// mesh (Springs::create_neigh + CSR_spring, src/spring.cpp:30-79,286-353,374-391):
//   structure list: for every face (f0, f1, f2) in order, append f1, f2 to row f0,
//                   f0, f2 to row f1 and f0, f1 to row f2, skipping neighbours
//                   already present;
//   bend list:      for every edge shared by two faces, the two vertices opposite
//                   that edge are joined (appended to both rows, in the order the
//                   second face is met; edges of a third face pair with the first);
//   rest length:    sqrt(((dx*dx + dy*dy) + dz*dz)) of the initial positions.
// Edges are looked up in a hash map keyed by the ordered vertex pair, which gives
// the same pairing as the reference's std::map (the order of results depends only
// on the face order).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/visg_sim.h"

namespace {

inline uint64_t key(uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | b; }

void emit(const std::vector<std::vector<uint32_t>>& nb, const float* xyz, uint32_t* row, VisgSpring* ent,
          int32_t* count) {
    size_t c = 0;
    const size_t nv = nb.size();
    for (size_t i = 0; i < nv; ++i) {
        if (row) row[i] = (uint32_t)c;
        for (uint32_t j : nb[i]) {
            if (ent) {
                float dx = xyz[3 * j] - xyz[3 * i], dy = xyz[3 * j + 1] - xyz[3 * i + 1];
                float dz = xyz[3 * j + 2] - xyz[3 * i + 2];
                volatile float px = dx * dx, py = dy * dy, pz = dz * dz;  // no contraction
                volatile float s = px + py;
                s = s + pz;
                ent[c].end = (int32_t)j;
                ent[c].rest = std::sqrt((float)s);
            }
            ++c;
        }
    }
    if (row) row[nv] = (uint32_t)c;
    if (count) *count = (int32_t)c;
}

// the structure and bend lists of create_neigh (spring.cpp:286-353); `seam` are the
// extra structure springs of a multi-piece garment, appended after the faces' ones
int springs_impl(const float* xyz, int32_t nv, const uint32_t* tris, int32_t nt,
                 const std::vector<std::pair<uint32_t, uint32_t>>& seam, uint32_t* row0, VisgSpring* ent0,
                 int32_t* n0, uint32_t* row1, VisgSpring* ent1, int32_t* n1) {
    if (!xyz || nv <= 0 || (nt > 0 && !tris) || nt < 0) return VISG_ERR_INVALID_ARG;
    for (int64_t k = 0; k < 3 * (int64_t)nt; ++k)
        if (tris[k] >= (uint32_t)nv) return VISG_ERR_INVALID_ARG;
    std::vector<std::vector<uint32_t>> n1v(nv), n2v(nv);
    auto push_unique = [](std::vector<uint32_t>& a, uint32_t v) {
        for (uint32_t u : a)
            if (u == v) return;
        a.push_back(v);
    };
    for (int i = 0; i < nt; ++i) {
        const uint32_t* f = tris + 3 * (size_t)i;
        push_unique(n1v[f[0]], f[1]);
        push_unique(n1v[f[0]], f[2]);
        push_unique(n1v[f[1]], f[0]);
        push_unique(n1v[f[1]], f[2]);
        push_unique(n1v[f[2]], f[0]);
        push_unique(n1v[f[2]], f[1]);
    }
    std::unordered_map<uint64_t, uint32_t> edge;  // first face's opposite vertex of each edge
    edge.reserve((size_t)nt * 2);
    std::vector<std::pair<uint32_t, uint32_t>> pairs;
    auto insert = [&](uint32_t a, uint32_t b, uint32_t c) {
        auto it = edge.find(key(a, b));
        if (it == edge.end()) it = edge.find(key(b, a));
        if (it != edge.end()) {
            pairs.push_back({it->second, c});
            return;
        }
        edge.emplace(key(a, b), c);
    };
    for (int i = 0; i < nt; ++i) {
        const uint32_t* f = tris + 3 * (size_t)i;
        insert(f[0], f[1], f[2]);
        insert(f[0], f[2], f[1]);
        insert(f[1], f[2], f[0]);
    }
    for (auto& pr : seam) n1v[pr.first].push_back(pr.second);
    for (auto& pr : pairs) {
        n2v[pr.first].push_back(pr.second);
        n2v[pr.second].push_back(pr.first);
    }
    emit(n1v, xyz, row0, ent0, n0);
    emit(n2v, xyz, row1, ent1, n1);
    return VISG_OK;
}

}  // namespace

namespace visg {
int sewing_pairs(const float* xyz, int64_t n, const int32_t* sizes, int32_t n_groups,
                 std::vector<std::pair<uint32_t, uint32_t>>& out, std::string& err);  // visg_mesh.cpp
void set_last_error(const char* msg);                                               // visg_api.cu
}  // namespace visg

extern "C" int visg_springs_from_mesh(const float* xyz, int32_t nv, const uint32_t* tris, int32_t nt, uint32_t* row0,
                                      VisgSpring* ent0, int32_t* n0, uint32_t* row1, VisgSpring* ent1, int32_t* n1) {
    return springs_impl(xyz, nv, tris, nt, {}, row0, ent0, n0, row1, ent1, n1);
}

extern "C" int visg_springs_from_mesh_sewn(const float* xyz, int32_t nv, const uint32_t* tris, int32_t nt,
                                           const int32_t* group_sizes, int32_t n_groups, uint32_t* row0,
                                           VisgSpring* ent0, int32_t* n0, uint32_t* row1, VisgSpring* ent1,
                                           int32_t* n1) {
    if (!xyz || nv <= 0 || !group_sizes) return VISG_ERR_INVALID_ARG;
    std::vector<std::pair<uint32_t, uint32_t>> seam;
    std::string err;
    if (visg::sewing_pairs(xyz, nv, group_sizes, n_groups, seam, err)) {
        visg::set_last_error(err.c_str());
        return VISG_ERR_INVALID_ARG;
    }
    return springs_impl(xyz, nv, tris, nt, seam, row0, ent0, n0, row1, ent1, n1);
}
