// Sanitizer driver for the host mesh code (OBJ reader, mesh transforms, spring and
// seam builders), built and run by tests/test_fuzz_mesh.py with AddressSanitizer and
// UBSan: every OBJ path given on the command line, then mutations of a small
// multi-piece OBJ, then random triangle soups with out-of-range indices and random
// vertex groups.  Exits non-zero (or the sanitizers abort) on any defect.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "../include/visg_sim.h"

namespace visg {
void set_last_error(const char*) {}  // the library's error text lives in visg_api.cu
}

static int springs(const std::vector<float>& xyz, const std::vector<uint32_t>& tris, const std::vector<int32_t>* groups) {
    const int32_t nv = (int32_t)(xyz.size() / 3), nt = (int32_t)(tris.size() / 3);
    int32_t n0 = 0, n1 = 0;
    auto call = [&](uint32_t* r0, VisgSpring* e0, uint32_t* r1, VisgSpring* e1) {
        return groups ? visg_springs_from_mesh_sewn(xyz.data(), nv, tris.data(), nt, groups->data(),
                                                    (int32_t)groups->size(), r0, e0, &n0, r1, e1, &n1)
                      : visg_springs_from_mesh(xyz.data(), nv, tris.data(), nt, r0, e0, &n0, r1, e1, &n1);
    };
    if (call(nullptr, nullptr, nullptr, nullptr) != 0) return 0;
    std::vector<uint32_t> r0((size_t)nv + 1), r1((size_t)nv + 1);
    std::vector<VisgSpring> e0((size_t)n0 + 1), e1((size_t)n1 + 1);
    if (call(r0.data(), e0.data(), r1.data(), e1.data()) != 0) return 1;
    for (int32_t k = 0; k < n0; ++k)
        if (e0[k].end < 0 || e0[k].end >= nv) return 1;
    for (int32_t k = 0; k < n1; ++k)
        if (e1[k].end < 0 || e1[k].end >= nv) return 1;
    return 0;
}

static int obj(const char* path) {
    VisgObj* o = nullptr;
    int32_t nv = 0, nf = 0;
    if (visg_obj_load(path, &o, &nv, &nf) != 0) return 0;  // rejected: fine
    std::vector<float> xyz(3 * (size_t)nv + 1), nrm(3 * (size_t)nv + 1);
    std::vector<uint32_t> f(3 * (size_t)nf + 1);
    int bad = visg_obj_get(o, xyz.data(), nrm.data(), f.data()) != 0;
    for (int32_t k = 0; k < 3 * nf; ++k)
        if (f[k] >= (uint32_t)nv) bad = 1;
    int32_t ng = 0;
    visg_obj_groups(o, nullptr, &ng);
    std::vector<int32_t> g((size_t)ng + 1);
    visg_obj_groups(o, g.data(), &ng);
    g.resize((size_t)ng);
    if (nv > 0) {
        visg_mesh_scale(xyz.data(), nv, 1.5f);
        visg_mesh_translate(xyz.data(), nv, 0.1f, 0.2f, 0.3f);
        visg_mesh_rotate(xyz.data(), nv, 33.0f, 1);
    }
    xyz.resize(3 * (size_t)nv);
    f.resize(3 * (size_t)nf);
    if (nv > 0) {
        bad |= springs(xyz, f, nullptr);
        if (ng >= 2 && ng % 2 == 0) bad |= springs(xyz, f, &g);
    }
    visg_obj_free(o);
    return bad;
}

int main(int argc, char** argv) {
    int bad = 0;
    for (int a = 2; a < argc; ++a) bad |= obj(argv[a]);
    const std::string tmp = argc > 1 ? argv[1] : "fuzz.obj";
    const char* base =
        "# object piece0\n# 4 vertices\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n"
        "f 2/1/1 4/1/1 3/1/1\n# object piece0_boundary\n# 1 vertices\nv 1 1 0.1\n# object piece1\n"
        "# 3 vertices\nv 2 0 0\nv 3 0 0\nv 2 1 0\nf 5 6 7\n# object piece1_boundary\n# 1 vertices\nv 2 1 0.1\n";
    const char* toks[] = {"v", "vn", "f", "#", "-1", "0", "99999", "1/", "//", "/1", "nan", "inf", "1e40", "\n",
                          " ", "x", "mtllib", "# object", "vertices", "2147483647", "-2147483648", "3/3/3"};
    std::mt19937 rng(1);
    for (int it = 0; it < 2000; ++it) {
        std::string s = base;
        const int nm = 1 + (int)(rng() % 6);
        for (int m = 0; m < nm; ++m) {
            const size_t pos = rng() % (s.size() + 1);
            if (rng() % 3 == 0 && !s.empty())
                s.erase(pos < s.size() ? pos : s.size() - 1, 1 + rng() % 4);
            else
                s.insert(pos < s.size() ? pos : s.size(),
                         std::string(toks[rng() % (sizeof toks / sizeof *toks)]) + (rng() % 2 ? " " : ""));
        }
        FILE* fp = std::fopen(tmp.c_str(), "w");
        if (!fp) return 2;
        std::fwrite(s.data(), 1, s.size(), fp);
        std::fclose(fp);
        bad |= obj(tmp.c_str());
    }
    for (int it = 0; it < 1000; ++it) {
        const int nv = 1 + (int)(rng() % 60), nt = (int)(rng() % 80);
        std::vector<float> xyz(3 * (size_t)nv);
        for (auto& v : xyz) v = (float)(rng() % 5) * 0.1f;  // many coincident points
        std::vector<uint32_t> t(3 * (size_t)nt);
        for (auto& v : t) v = rng() % (uint32_t)(nv + (it % 7 == 0 ? 2 : 0));  // some out of range
        bad |= springs(xyz, t, nullptr);
        std::vector<int32_t> g;
        int left = nv;
        while (left > 0 && g.size() < 6) {
            const int a = 1 + (int)(rng() % left);
            g.push_back(a);
            left -= a;
        }
        if (g.size() % 2) g.push_back(0);
        bad |= springs(xyz, t, &g);
    }
    std::printf("fuzz_mesh: %s\n", bad ? "DEFECT" : "clean");
    return bad;
}
