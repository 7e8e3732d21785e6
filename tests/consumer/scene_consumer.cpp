// scene_consumer.cpp — a C++ host program that drives the library through its C
// ABI alone (include/visg_sim.h, -lvisgsim), the way the reference's Scene drives
// its Simulator:
//   Scene::init_simulation (scene.cpp:176-186): meshes from OBJ files, the
//     reference's spring lists from the cloth's triangles, the reference's
//     constants, the simulator over the body;
//   Scene::RenderGPU_CUDA (scene.cpp:267-276): one step per frame, then the output
//     stage (positions as vec4 and per-vertex normals of the pre-step positions);
//   Scene::OnMouseMove (scene.cpp:357): one vertex dragged on a given frame;
//   Scene::~Scene (scene.cpp:85): the simulator destroyed.
// Writes the final positions, the last frame's pos4 and vertex normals to a binary
// file:  int32 n, float x[3n], float pos4[4n], float normals[3n].
//
// usage: scene_consumer cloth.obj body.obj frames drag_frame drag_vertex dy out.bin
// exit status: 0 ok, 2 a library call failed (the message is printed), 1 bad usage.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "visg_sim.h"

namespace {

struct Mesh {
    int nv = 0, nf = 0;
    std::vector<float> xyz, normals;
    std::vector<uint32_t> faces;
};

bool ok(int status, const char* what) {
    if (status == VISG_OK) return true;
    std::fprintf(stderr, "%s failed (%d): %s\n", what, status, visg_last_error());
    return false;
}

bool load(const char* path, Mesh& m) {
    VisgObj* obj = nullptr;
    if (!ok(visg_obj_load(path, &obj, &m.nv, &m.nf), "visg_obj_load")) return false;
    m.xyz.resize(3 * (size_t)m.nv);
    m.normals.resize(3 * (size_t)m.nv);
    m.faces.resize(3 * (size_t)m.nf);
    const bool good = ok(visg_obj_get(obj, m.xyz.data(), m.normals.data(), m.faces.data()), "visg_obj_get");
    visg_obj_free(obj);
    return good;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s cloth.obj body.obj frames drag_frame drag_vertex dy out.bin\n", argv[0]);
        return 1;
    }
    const int frames = std::atoi(argv[3]), drag_frame = std::atoi(argv[4]);
    const uint32_t drag_vertex = (uint32_t)std::atoi(argv[5]);
    const float dy = (float)std::atof(argv[6]);

    // ---- Scene::init_simulation --------------------------------------------------------
    Mesh cloth, body;
    if (!load(argv[1], cloth) || !load(argv[2], body)) return 2;
    const int N = cloth.nv;
    int32_t n0 = 0, n1 = 0;
    if (!ok(visg_springs_from_mesh(cloth.xyz.data(), N, cloth.faces.data(), cloth.nf, nullptr, nullptr, &n0, nullptr,
                                   nullptr, &n1),
            "visg_springs_from_mesh (counts)"))
        return 2;
    std::vector<uint32_t> r0(N + 1), r1(N + 1);
    std::vector<VisgSpring> e0(n0), e1(n1);
    if (!ok(visg_springs_from_mesh(cloth.xyz.data(), N, cloth.faces.data(), cloth.nf, r0.data(), e0.data(), &n0,
                                   r1.data(), e1.data(), &n1),
            "visg_springs_from_mesh"))
        return 2;
    const uint32_t* rows[2] = {r0.data(), r1.data()};
    const VisgSpring* csr[2] = {e0.data(), e1.data()};
    VisgParams p;
    visg_default_params(&p);  // the reference's constants
    VisgSim* sim = nullptr;
    if (!ok(visg_create(&p, cloth.xyz.data(), N, rows, csr, nullptr, body.xyz.data(), body.normals.data(), body.nv,
                        body.faces.data(), body.nf, &sim),
            "visg_create"))
        return 2;
    if (!ok(visg_set_faces(sim, cloth.faces.data(), cloth.nf), "visg_set_faces")) return 2;

    // ---- Scene::RenderGPU_CUDA per frame, Scene::OnMouseMove once --------------------------
    std::vector<float> x(3 * (size_t)N), pos4(4 * (size_t)N), vn(3 * (size_t)N);
    for (int f = 0; f < frames; ++f) {
        if (f == drag_frame) {
            if (!ok(visg_get_positions(sim, x.data(), 0), "visg_get_positions")) return 2;
            const float target[3] = {x[3 * drag_vertex], x[3 * drag_vertex + 1] + dy, x[3 * drag_vertex + 2]};
            if (!ok(visg_set_vertex(sim, drag_vertex, target), "visg_set_vertex")) return 2;
        }
        if (!ok(visg_step(sim, 1), "visg_step")) return 2;
        if (!ok(visg_render(sim, pos4.data(), vn.data(), nullptr, 0, 1), "visg_render")) return 2;
    }
    if (!ok(visg_get_positions(sim, x.data(), 0), "visg_get_positions")) return 2;
    int64_t contacts = 0;
    if (!ok(visg_count_contacts(sim, &contacts), "visg_count_contacts")) return 2;

    // ---- Scene::~Scene ---------------------------------------------------------------------
    if (!ok(visg_destroy(sim), "visg_destroy")) return 2;

    FILE* out = std::fopen(argv[7], "wb");
    if (!out) {
        std::fprintf(stderr, "cannot write %s\n", argv[7]);
        return 2;
    }
    const int32_t n = N;
    std::fwrite(&n, 4, 1, out);
    std::fwrite(x.data(), 4, x.size(), out);
    std::fwrite(pos4.data(), 4, pos4.size(), out);
    std::fwrite(vn.data(), 4, vn.size(), out);
    std::fclose(out);
    std::printf("%d vertices, %d springs, %d frames, %lld in contact\n", N, n0 + n1, frames, (long long)contacts);
    return 0;
}
