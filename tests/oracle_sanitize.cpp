// Sanitizer driver for the oracle (the CPU restatement the parity tests check
// against), built and run by tests/test_fuzz_mesh.py with AddressSanitizer and UBSan:
// float and FP64 simulators over a grid sheet with a sphere, a single triangle, no
// body and a duplicated triangle; steps, body updates, pins, vertex updates, state
// round trips, LBVH export, queries, the FP64 adjoint, the output stage and shading.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include "../include/visg_sim.h"
extern "C" {
void* orc_sim_create(int prec, const VisgParams* p, const float* cloth, int N, const uint32_t* const* rows,
                     const VisgSpring* const* ents, const float* const* ks, const float* body, const float* bn,
                     int nv, const uint32_t* tris, int nt);
void orc_sim_destroy(void*); void orc_sim_step(void*, int); void orc_sim_update_body(void*, const float*, const float*);
void orc_sim_set_vertex(void*, int, const float*); void orc_sim_set_pinned(void*, const uint32_t*, int);
void orc_sim_get_state(void*, double*, double*, double*); void orc_sim_set_state(void*, const float*, const float*, const float*);
int orc_sim_n_leaves(void*);
void orc_sim_export_lbvh(void*, uint32_t*, float*, uint32_t*, int32_t*, int32_t*, int32_t*, int32_t*, int32_t*, float*, float*, float*);
void orc_sim_query(void*, const float*, int, int32_t*, int32_t*, double*, double*);
int orc_sim_forward(void*, int, int, void**); void orc_sim_backward(void*, void*, const double*, const double*, double*, double*);
void orc_render(const float*, const float*, int, const uint32_t*, int, float*, float*, float*);
void orc_sh_shade(const float*, int, const float*, float*);
int orc_springs_from_mesh(const float*, int, const uint32_t*, int, uint32_t*, VisgSpring*, int*, uint32_t*, VisgSpring*, int*);
}
// the reference's constants (the library's visg_default_params, which this driver does not link)
void visg_default_params(VisgParams* p) {
    std::memset(p, 0, sizeof *p); p->dt = 1.0f / 40; p->mass = 0.3f; p->gravity[1] = -0.00981f; p->force_damping = -0.02f;
    p->spring_damping = -0.5f; p->verlet_damping = 1.0f; p->thickness = 0.003f; p->box_depth = 0.01f; p->n_lists = 2;
    p->list_k[0] = 100; p->list_k[1] = 2; p->collide = 1; p->max_displacement = 1; p->use_graph = 1; p->split_collision = 1; p->collision_margin = 1;
}
static void sphere(int nu, int nvv, float r, float cy, std::vector<float>& xyz, std::vector<float>& nrm, std::vector<uint32_t>& tri) {
    for (int i = 0; i <= nvv; ++i) for (int j = 0; j < nu; ++j) {
        float th = 3.14159265f * i / nvv, ph = 6.2831853f * j / nu;
        float x = std::sin(th) * std::cos(ph), y = std::cos(th), z = std::sin(th) * std::sin(ph);
        xyz.insert(xyz.end(), {r * x, cy + r * y, r * z}); nrm.insert(nrm.end(), {x, y, z});
    }
    for (int i = 0; i < nvv; ++i) for (int j = 0; j < nu; ++j) {
        uint32_t a = i * nu + j, b = i * nu + (j + 1) % nu, c = (i + 1) * nu + j, d = (i + 1) * nu + (j + 1) % nu;
        tri.insert(tri.end(), {a, c, b, b, c, d});
    }
}
int main() {
    const int n = 24, N = n * n;
    std::vector<float> cloth; std::vector<uint32_t> ct;
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) cloth.insert(cloth.end(), {j / (float)(n - 1) - 0.5f, 0.0f, i / (float)(n - 1) - 0.5f});
    for (int i = 0; i + 1 < n; ++i) for (int j = 0; j + 1 < n; ++j) { uint32_t a = i * n + j; ct.insert(ct.end(), {a, a + 1, a + (uint32_t)n, a + 1, a + n + 1, a + (uint32_t)n}); }
    int n0 = 0, n1 = 0;
    orc_springs_from_mesh(cloth.data(), N, ct.data(), (int)ct.size() / 3, nullptr, nullptr, &n0, nullptr, nullptr, &n1);
    std::vector<uint32_t> r0(N + 1), r1(N + 1); std::vector<VisgSpring> e0(n0 + 1), e1(n1 + 1);
    orc_springs_from_mesh(cloth.data(), N, ct.data(), (int)ct.size() / 3, r0.data(), e0.data(), &n0, r1.data(), e1.data(), &n1);
    const uint32_t* rows[2] = {r0.data(), r1.data()}; const VisgSpring* ents[2] = {e0.data(), e1.data()};
    std::vector<float> bx, bn; std::vector<uint32_t> bt;
    sphere(16, 12, 0.3f, -0.31f, bx, bn, bt);
    VisgParams p; visg_default_params(&p);
    for (int prec : {4, 8}) for (int variant = 0; variant < 4; ++variant) {
        int nt = variant == 0 ? (int)bt.size() / 3 : variant == 1 ? 1 : variant == 2 ? 0 : 2;
        std::vector<uint32_t> tris(bt.begin(), bt.begin() + 3 * nt);
        if (variant == 3) { tris[3] = tris[0]; tris[4] = tris[1]; tris[5] = tris[2]; }  // a duplicate triangle
        void* s = orc_sim_create(prec, &p, cloth.data(), N, rows, ents, nullptr, nt ? bx.data() : nullptr, nt ? bn.data() : nullptr,
                                 nt ? (int)bx.size() / 3 : 0, nt ? tris.data() : nullptr, nt);
        uint32_t pins[2] = {0, (uint32_t)n - 1}; orc_sim_set_pinned(s, pins, 2);
        orc_sim_step(s, 60);
        std::vector<float> moved(bx); for (size_t k = 1; k < moved.size(); k += 3) moved[k] += 0.01f;
        if (nt) orc_sim_update_body(s, moved.data(), bn.data());
        orc_sim_step(s, 20);
        float v[3] = {0.1f, 0.2f, 0.0f}; orc_sim_set_vertex(s, 5, v);
        std::vector<double> x(3 * N), xo(3 * N), nn(3 * N); orc_sim_get_state(s, x.data(), xo.data(), nn.data());
        std::vector<float> xf(x.begin(), x.end()), xof(xo.begin(), xo.end()), nf(nn.begin(), nn.end());
        orc_sim_set_state(s, xf.data(), xof.data(), nf.data());
        if (nt) {
            int T = nt, L = orc_sim_n_leaves(s);
            std::vector<uint32_t> tc(T), sc(T); std::vector<float> tb(6 * T), ib(6 * T), lb(6 * T), rb(6);
            std::vector<int32_t> st(T), ca(T), cb(T), pi(T), pl(T);
            orc_sim_export_lbvh(s, tc.data(), tb.data(), sc.data(), st.data(), ca.data(), cb.data(), pi.data(), pl.data(), ib.data(), lb.data(), rb.data());
            (void)L;
            std::vector<float> pts; std::mt19937 rng(3); for (int k = 0; k < 300; ++k) pts.push_back((rng() % 1000) / 1000.0f - 0.5f);
            std::vector<int32_t> leaf(100), in(100); std::vector<double> dist(100), qn(300);
            orc_sim_query(s, pts.data(), 100, leaf.data(), in.data(), dist.data(), qn.data());
        }
        if (prec == 8 && variant == 0) {
            void* tape = nullptr; orc_sim_forward(s, 30, 8, &tape);
            std::vector<double> dl(3 * N, 1e-3), dk(n0 + n1 + 1), ds(3);
            orc_sim_backward(s, tape, dl.data(), nullptr, dk.data(), ds.data());
        }
        orc_sim_destroy(s);
    }
    std::vector<float> pos4(4 * N), vn(3 * N), fn(3 * ct.size() / 3), col(3 * N); float rgb[3] = {1, 0.5f, 0.25f};
    orc_render(cloth.data(), cloth.data(), N, ct.data(), (int)ct.size() / 3, pos4.data(), vn.data(), fn.data());
    orc_sh_shade(vn.data(), N, rgb, col.data());
    std::printf("oracle_sanitize: clean\n");
}
