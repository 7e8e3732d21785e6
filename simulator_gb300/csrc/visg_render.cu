// visg_render.cu — the output stage of a step, headless.
//
// The reference's Simulator::cuda_update_vbo (src/simulation.cu:196-231) writes the
// step's positions into the GL vertex buffer (update_vbo_pos, verlet.cu:119-127),
// then per-face normals (compute_face_normal, verlet.cu:91-116) of the positions the
// step started from, then per-vertex normals as the normalised sum of the adjacent
// faces' normals in face order (compute_vbo_normal, verlet.cu:163-181, over the
// vertex -> face CSR of get_vertex_adjface, simulation.cu:152-180).  Here the GL
// buffers become caller buffers (device or host); the arithmetic is the reference's,
// one IEEE rounding per operation (cross, normalize as GLM 0.9.9.8 defines them), so
// the results are bit-identical to the reference's kernels.
//
// All three are gather/stream kernels bounded by HBM: per vertex 16 B read + 16 B
// written (positions), per face 3 gathered 16-B position reads + 12 B written, per
// vertex 4 B row + 4 B per adjacent face + the gathered face normals (12 B each,
// mostly L2 hits) + 12 B written (+ 12 B of shaded colour when asked for).
#include <cuda_runtime.h>
#include <stdint.h>

#include "visg_internal.cuh"

namespace visg {

namespace {

constexpr int RENDER_THREADS = 256;

// pos4[i] = (x, y, z, 1): glm::vec4(pos, 1.0) of update_vbo_pos
__global__ void __launch_bounds__(RENDER_THREADS) k_render_pos(const float4* __restrict__ st, int64_t n,
                                                               float4* __restrict__ pos4) {
    const int64_t i = (int64_t)blockIdx.x * RENDER_THREADS + threadIdx.x;
    if (i >= n) return;
    const float4 s = __ldg(st + 2 * i);
    pos4[i] = make_float4(s.x, s.y, s.z, 1.0f);
}

// fn[f] = normalize(cross(p1 - p0, p2 - p0)) of the positions in records st
__global__ void __launch_bounds__(RENDER_THREADS) k_face_normals(const float4* __restrict__ st,
                                                                 const uint32_t* __restrict__ faces, int64_t nf,
                                                                 float* __restrict__ fn) {
    const int64_t f = (int64_t)blockIdx.x * RENDER_THREADS + threadIdx.x;
    if (f >= nf) return;
    const uint32_t a = __ldg(faces + 3 * f), b = __ldg(faces + 3 * f + 1), c = __ldg(faces + 3 * f + 2);
    const f3 p0 = xyz(__ldg(st + 2 * (int64_t)a));
    const f3 p1 = xyz(__ldg(st + 2 * (int64_t)b));
    const f3 p2 = xyz(__ldg(st + 2 * (int64_t)c));
    const f3 nrm = normalize(cross(sub(p1, p0), sub(p2, p0)));
    fn[3 * f] = nrm.x;
    fn[3 * f + 1] = nrm.y;
    fn[3 * f + 2] = nrm.z;
}

// Diffuse irradiance of the reference's fragment shader (src/shaders/sh.frag:13-55):
// the order-2 spherical-harmonic polynomial of Ramamoorthi & Hanrahan's irradiance
// environment map with the "old town square" coefficients, evaluated per vertex on
// the normalised normal, term by term in the shader's order (its L21 term uses
// x*y, as written there), times the object colour; ambient and specular are zero
// and the texture lookup is dropped.
__device__ __forceinline__ f3 sh_colour(f3 v, f3 rgb) {
    constexpr float C1 = 0.429043f, C2 = 0.511664f, C3 = 0.743125f, C4 = 0.886227f, C5 = 0.247708f;
    const f3 L00 = mk3(0.87f, 0.87f, 0.86f), L1m1 = mk3(0.17f, 0.24f, 0.31f), L10 = mk3(0.03f, 0.03f, 0.03f);
    const f3 L11 = mk3(-0.004f, -0.03f, -0.05f), L2m2 = mk3(-0.12f, -0.12f, -0.11f);
    const f3 L2m1 = mk3(0.003f, 0.003f, 0.007f), L20 = mk3(-0.03f, -0.02f, -0.02f);
    const f3 L21 = mk3(-0.08f, -0.08f, -0.09f), L22 = mk3(-0.16f, -0.19f, -0.22f);
    const f3 t = normalize(v);
    const float c1x2 = __fmul_rn(2.0f, C1), c2x2 = __fmul_rn(2.0f, C2);
    f3 d = mul(mul(C1, L22), __fsub_rn(__fmul_rn(t.x, t.x), __fmul_rn(t.y, t.y)));
    d = add(d, mul(mul(mul(C3, L20), t.z), t.z));
    d = add(d, mul(C4, L00));
    d = sub(d, mul(C5, L20));
    d = add(d, mul(mul(mul(c1x2, L2m2), t.x), t.y));
    d = add(d, mul(mul(mul(c1x2, L21), t.x), t.y));
    d = add(d, mul(mul(mul(c1x2, L2m1), t.y), t.z));
    d = add(d, mul(mul(c2x2, L11), t.x));
    d = add(d, mul(mul(c2x2, L1m1), t.y));
    d = add(d, mul(mul(c2x2, L10), t.z));
    d = mul(d, 1.0f);  // scaleColor
    const f3 r = add(add(mk3(0.0f, 0.0f, 0.0f), d), mk3(0.0f, 0.0f, 0.0f));  // ambient + diffuse + specular
    return mk3(__fmul_rn(r.x, rgb.x), __fmul_rn(r.y, rgb.y), __fmul_rn(r.z, rgb.z));
}

// vn[i] = normalize(+0 + fn[f_0] + fn[f_1] + ...) over the vertex's faces in face order;
// with colours, also the shaded colour of that normal
__global__ void __launch_bounds__(RENDER_THREADS) k_vertex_normals(const uint32_t* __restrict__ row,
                                                                   const uint32_t* __restrict__ col,
                                                                   const float* __restrict__ fn, int64_t n,
                                                                   float* __restrict__ vn, float* __restrict__ colour,
                                                                   const f3 rgb) {
    const int64_t i = (int64_t)blockIdx.x * RENDER_THREADS + threadIdx.x;
    if (i >= n) return;
    f3 s = mk3(0.0f, 0.0f, 0.0f);
    const uint32_t e1 = __ldg(row + i + 1);
    for (uint32_t e = __ldg(row + i); e < e1; ++e) {
        const uint32_t f = __ldg(col + e);
        s = add(s, mk3(__ldg(fn + 3 * (int64_t)f), __ldg(fn + 3 * (int64_t)f + 1), __ldg(fn + 3 * (int64_t)f + 2)));
    }
    const f3 v = normalize(s);
    if (vn) {
        vn[3 * i] = v.x;
        vn[3 * i + 1] = v.y;
        vn[3 * i + 2] = v.z;
    }
    if (colour) {
        const f3 c = sh_colour(v, rgb);
        colour[3 * i] = c.x;
        colour[3 * i + 1] = c.y;
        colour[3 * i + 2] = c.z;
    }
}

inline unsigned blocks_for(int64_t n) { return (unsigned)((n + RENDER_THREADS - 1) / RENDER_THREADS); }

}  // namespace

cudaError_t launch_render(const float4* st_now, const float4* st_prev, int64_t n, const uint32_t* faces, int64_t nf,
                          const uint32_t* row, const uint32_t* col, float* fn, float4* pos4, float* vn, float* colour,
                          const float* rgb, cudaStream_t s) {
    if (pos4 && n > 0) k_render_pos<<<blocks_for(n), RENDER_THREADS, 0, s>>>(st_now, n, pos4);
    if (fn && nf > 0) k_face_normals<<<blocks_for(nf), RENDER_THREADS, 0, s>>>(st_prev, faces, nf, fn);
    const f3 c = rgb ? f3{rgb[0], rgb[1], rgb[2]} : f3{1.0f, 1.0f, 1.0f};
    if ((vn || colour) && n > 0)
        k_vertex_normals<<<blocks_for(n), RENDER_THREADS, 0, s>>>(row, col, fn, n, vn, colour, c);
    return cudaGetLastError();
}

}  // namespace visg
