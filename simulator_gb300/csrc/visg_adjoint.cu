// visg_adjoint.cu — reverse-mode derivative of the fused step.
//
// One step (verlet.cu:129-161), for a vertex i that is not pinned:
//   v   = (x - xo)/dt
//   F   = m g + c v + sum_e f_e,  f_e = s_e u_e,  d_e = x_i - x_j + eps, L = |d_e|,
//         u_e = d_e/L, s_e = -k_e (L - L0_e) + kd (v_i - v_j).u_e
//   F*  = F - (n.F) n                       (n = contact normal entering the step, frozen)
//   X*  = x + gamma (x - xo) + F*/m dt^2    (gamma = 1: the reference's 2x - xo + a dt^2)
//   contact (frozen active set, plane normal nu):  X = X* - ((X* - p0).nu) nu,  XO = X
//   no contact:                                    X = X*,                      XO = x
// Pinned: X = XO = x.  Given the adjoints (lX, lXO) of a step's outputs, the step's
// inputs receive
//   l*  = Q (lX + lXO) with Q = I - nu nu^T (contact), or l* = lX and lx += lXO
//   lx += (1 + gamma) l*,  lxo -= gamma l*,  dL/dgamma += l*.(x - xo)
//   G   = P (dt^2/m) l*  with P = I - n n^T    (adjoint of the force on i)
//   lx += (c/dt) G, lxo -= (c/dt) G,  dL/dc += G.v
//   every spring e = (i -> j) with adjoint G_i adds to x_i, xo_i and (negated) x_j, xo_j,
//   and dL/dk_e += -(L - L0) u.G_i,  dL/dkd += (dv.u)(u.G_i).
// k_adj_self does everything owned by vertex i (no atomics); k_adj_gather adds the
// x_j / xo_j terms by walking j's row and looking up each spring's reverse entry.
//
// The differentiated trajectory is computed in FP64 (k_step_f64, the same algorithm
// in double, traversing the body's float LBVH with the double position): stiff
// springs stretch by ~1e-6 of the cloth's size, about the resolution of float
// positions, so gradients with respect to stiffness along a float trajectory carry
// percent-level noise.  The contact set the FP64 forward finds is frozen for the
// reverse sweep.
#include <cuda_runtime.h>
#include <stdint.h>

#include "visg_internal.cuh"

namespace visg {

namespace {

// The reverse sweep runs in double: per-spring contributions of both signs cancel
// over hundreds of steps, and float accumulation loses several digits there (the
// forward trajectory it differentiates is the float one, bit for bit).
struct V {
    double x, y, z;
};
__device__ __forceinline__ V ld3(const float* p, int64_t i) { return V{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ V ld3(const double* p, int64_t i) { return V{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ void st3(double* p, int64_t i, V v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
__device__ __forceinline__ V operator+(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V operator-(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V operator*(double s, V a) { return V{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dotv(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

constexpr double kEps = 1.1920928955078125e-07;

// derivative of spring e = (i -> j) contracted with G: returns the contributions to
// x_i and xo_i (those to x_j, xo_j are their negatives), dF/dk.G and dF/dkd.G
__device__ __forceinline__ void spring_adj(V xi, V xoi, V xj, V xoj, double k, double L0, double kd, double dt, V G,
                                           V& gx, V& gxo, double& gk, double& gkd) {
    const V vi = (1.0 / dt) * (xi - xoi), vj = (1.0 / dt) * (xj - xoj);
    const V d = (xi - xj) + V{kEps, kEps, kEps};
    const V dv = vi - vj;
    const double L = sqrt(dotv(d, d));
    const V u = (1.0 / L) * d;
    const double dvu = dotv(dv, u);
    const double s = -k * (L - L0) + kd * dvu;
    const double uG = dotv(u, G);
    const V dsdd = (-k) * u + (kd / L) * (dv - dvu * u);
    const V gd = uG * dsdd + (s / L) * (G - uG * u);
    const V gdv = (kd * uG) * u;
    gx = gd + (1.0 / dt) * gdv;
    gxo = (-1.0 / dt) * gdv;
    gk = -(L - L0) * uG;
    gkd = dvu * uG;
}

__device__ __forceinline__ float list_k(const StepParams& p, uint32_t word) {
    const int f = (int)(word >> LIST_SHIFT);
    return p.list_k[f & 3];
}

__device__ __forceinline__ void block_add3(double a, double b, double c, double* out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0 && (a != 0.0 || b != 0.0 || c != 0.0)) {
        atomicAdd(&out[0], a);
        atomicAdd(&out[1], b);
        atomicAdd(&out[2], c);
    }
}

__device__ __forceinline__ bool in_box_d(V p, float4 lo, float4 hi) {
    return (p.x >= (double)lo.x && p.x <= (double)hi.x) && (p.y >= (double)lo.y && p.y <= (double)hi.y) &&
           (p.z >= (double)lo.z && p.z <= (double)hi.z);
}

// first-hit traversal (cudaBRT.cu:239-285) of the float tree for a double point
__device__ int first_hit_d(const BvhView& bv, V p, int* err) {
    const int nl = bv.root->n_leaves;
    if (nl <= 0 || !in_box_d(p, bv.root->top_lo, bv.root->top_hi)) return -1;
    if (nl == 1) return 0;
    int stack[32];
    int sp = 0, node = bv.root->root, budget = nl;
    while (true) {
        if (--budget < 0) {
            atomicOr(err, ERR_STACK);
            return -1;
        }
        const Node& nd = bv.nodes[node];
        const int la = __float_as_int(nd.a_lo.w), lb = __float_as_int(nd.b_lo.w);
        const bool ol = in_box_d(p, nd.a_lo, nd.a_hi), orr = in_box_d(p, nd.b_lo, nd.b_hi);
        if (ol && la < 0) return ~la;
        if (orr && lb < 0) return ~lb;
        const bool tl = ol && la >= 0, tr = orr && lb >= 0;
        if (!tl && !tr) {
            if (sp == 0) return -1;
            node = stack[--sp];
        } else {
            node = tl ? la : lb;
            if (tl && tr) {
                if (sp == 32) {
                    atomicOr(err, ERR_STACK);
                    return -1;
                }
                stack[sp++] = lb;
            }
        }
    }
}

// One step in double, operation by operation the FP64 oracle's arithmetic (the
// reference's expressions evaluated in double with one rounding per operation), so
// the GPU's differentiable trajectory and contact set equal the oracle's bit for bit.
struct R {
    double x, y, z;
};
__device__ __forceinline__ R radd(R a, R b) { return R{__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)}; }
__device__ __forceinline__ R rsub(R a, R b) { return R{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
__device__ __forceinline__ R rmul(R a, double s) { return R{__dmul_rn(a.x, s), __dmul_rn(a.y, s), __dmul_rn(a.z, s)}; }
__device__ __forceinline__ R rmul(double s, R a) { return R{__dmul_rn(s, a.x), __dmul_rn(s, a.y), __dmul_rn(s, a.z)}; }
__device__ __forceinline__ R rdiv(R a, double s) { return R{__ddiv_rn(a.x, s), __ddiv_rn(a.y, s), __ddiv_rn(a.z, s)}; }
__device__ __forceinline__ double rdot(R a, R b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ R rnormalize(R v) { return rmul(v, __ddiv_rn(1.0, __dsqrt_rn(rdot(v, v)))); }
__device__ __forceinline__ R rcross(R a, R b) {
    return R{__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(b.y, a.z)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(b.z, a.x)),
             __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(b.x, a.y))};
}
__device__ __forceinline__ R rld(const double* p, int64_t i) { return R{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ void rst(double* p, int64_t i, R v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
__device__ __forceinline__ R rf4(float4 v) { return R{v.x, v.y, v.z}; }

__global__ void k_step_f64(const double* __restrict__ x, const double* __restrict__ xo, double* __restrict__ xn_out,
                           double* __restrict__ xon_out, double* __restrict__ nrm, const uint32_t* __restrict__ rowp,
                           const uint2* __restrict__ ent, const float* __restrict__ kent, const BvhView* bodies,
                           const float4* __restrict__ body_verts, const uint32_t* __restrict__ body_tris,
                           const StepParams P, int refv, int collide, int n, int* err, unsigned* contacts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const R pos0 = rld(x, i), pold = rld(xo, i);
    const uint32_t rp0 = rowp[i];
    if (rp0 & PIN_BIT) {
        rst(xn_out, i, pos0);
        rst(xon_out, i, pos0);
        rst(nrm, i, R{0, 0, 0});
        return;
    }
    const double dt = P.dt, mass = P.mass, kd = P.kd, eps = kEps;
    const R vel = rdiv(rsub(pos0, pold), dt);
    R force = radd(rmul(R{P.gx, P.gy, P.gz}, mass), rmul(vel, (double)P.damp));
    R acc{0, 0, 0};
    int list = 0;
    const uint32_t re = rowp[i + 1] & ROW_MASK;
    for (uint32_t e = rp0 & ROW_MASK; e < re; ++e) {
        const uint2 en = ent[e];
        const int f = (int)(en.x >> LIST_SHIFT);
        while (list < f) {
            force = radd(force, acc);
            acc = R{0, 0, 0};
            ++list;
        }
        const int j = (int)(en.x & END_MASK);
        const double ks = kent ? (double)kent[e] : (double)P.list_k[f & 3];
        const R p2 = rld(x, j), p2o = rld(xo, j);
        const R v2 = rdiv(rsub(p2, p2o), dt);
        const R dP = radd(rsub(pos0, p2), R{eps, eps, eps});
        const R dV = rsub(vel, v2);
        const double dist = __dsqrt_rn(rdot(dP, dP));
        const double left = __dmul_rn(-ks, __dsub_rn(dist, (double)__uint_as_float(en.y)));
        const double right = __dmul_rn(kd, __ddiv_rn(rdot(dV, dP), dist));
        acc = radd(acc, rmul(__dadd_rn(left, right), rnormalize(dP)));
    }
    while (list < P.n_lists) {
        force = radd(force, acc);
        acc = R{0, 0, 0};
        ++list;
    }
    const R cf = rld(nrm, i);
    force = rsub(force, rmul(rdot(cf, force), cf));
    const R a = rdiv(force, mass);
    const R adt = rmul(rmul(a, dt), dt);
    R pos = refv ? radd(rsub(radd(pos0, pos0), pold), adt)
                 : radd(radd(pos0, rmul((double)P.gamma, rsub(pos0, pold))), adt);
    R pos_old = pos0;
    R nn{0, 0, 0};
    if (collide && bodies[0].root != nullptr) {
        const int leaf = first_hit_d(bodies[0], V{pos.x, pos.y, pos.z}, err);
        if (leaf >= 0) {
            const int t = __float_as_int(bodies[0].leaves[2 * leaf + 1].z);
            const R v0 = rf4(body_verts[body_tris[3 * t]]), v1 = rf4(body_verts[body_tris[3 * t + 1]]),
                    v2 = rf4(body_verts[body_tris[3 * t + 2]]);
            const R normal = rnormalize(rcross(rsub(v1, v0), rsub(v2, v0)));
            double dist = rdot(rsub(pos, v0), normal);
            if (!(dist > 0.0)) {
                dist = __dmul_rn(1.0, fabs(dist));
                pos = radd(pos, rmul(dist, normal));
                pos_old = pos;
                nn = normal;
            }
        }
    }
    rst(xn_out, i, pos);
    rst(xon_out, i, pos_old);
    rst(nrm, i, nn);
    if (contacts) {  // vertices projected in this step, one atomic per warp
        const unsigned act = __activemask();
        const unsigned m = __ballot_sync(act, nn.x != 0.0 || nn.y != 0.0 || nn.z != 0.0);
        if (m && (int)(threadIdx.x & 31u) == __ffs(act) - 1) atomicAdd(contacts, (unsigned)__popc(m));
    }
}

__global__ void k_widen(const float* __restrict__ src, double* __restrict__ dst, int64_t n) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = (double)src[k];
}

__global__ void k_narrow(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = (float)src[k];
}

__global__ void k_adj_self(const AdjArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < a.n;
    double dg = 0.0, dc = 0.0, dkd = 0.0;
    if (active) {
        const StepParams& P = a.p;
        const V lX = ld3(a.lx_in, i), lXO = ld3(a.lxo_in, i);
        const uint32_t rp0 = a.rowp[i];
        const bool pinned = (rp0 & PIN_BIT) != 0u;
        V lx{0, 0, 0}, lxo{0, 0, 0}, G{0, 0, 0};
        if (pinned) {
            lx = lX + lXO;
        } else {
            const V x = ld3(a.x, i), xo = ld3(a.xo, i);
            const V nu = ld3(a.n_out, i), np = ld3(a.n_in, i);
            V ls;
            if (nu.x != 0.0f || nu.y != 0.0f || nu.z != 0.0f) {
                const V s = lX + lXO;
                ls = s - dotv(nu, s) * nu;
            } else {
                ls = lX;
                lx = lx + lXO;
            }
            const double gam = P.gamma, dt = P.dt;
            lx = lx + (1.0 + gam) * ls;
            lxo = lxo - gam * ls;
            dg += dotv(ls, x - xo);
            const V h = (dt * dt / (double)P.mass) * ls;
            G = h - dotv(np, h) * np;
            const V v = (1.0 / dt) * (x - xo);
            dc += dotv(G, v);
            lx = lx + ((double)P.damp / dt) * G;
            lxo = lxo - ((double)P.damp / dt) * G;
            const uint32_t re = a.rowp[i + 1] & ROW_MASK;
            for (uint32_t e = rp0 & ROW_MASK; e < re; ++e) {
                const uint2 en = a.ent[e];
                const int j = (int)(en.x & END_MASK);
                const float k = a.kent ? a.kent[e] : list_k(P, en.x);
                V gx, gxo;
                double gk, gkd;
                spring_adj(x, xo, ld3(a.x, j), ld3(a.xo, j), k, __uint_as_float(en.y), P.kd, P.dt, G, gx, gxo, gk, gkd);
                lx = lx + gx;
                lxo = lxo + gxo;
                a.dk[e] += gk;
                dkd += gkd;
            }
        }
        st3(a.lx_out, i, lx);
        st3(a.lxo_out, i, lxo);
        st3(a.G, i, G);
    }
    block_add3(dg, dc, dkd, a.dscalar);
}

// x_j / xo_j terms: for every entry e' = (j -> i) of j's row, the reverse entry
// e = (i -> j) of i's row is evaluated with i's force adjoint G_i.
__global__ void k_adj_gather(const AdjArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    const StepParams& P = a.p;
    const uint32_t rp = a.rowp[j] & ROW_MASK, re = a.rowp[j + 1] & ROW_MASK;
    const V xj = ld3(a.x, j), xoj = ld3(a.xo, j);
    V lx = ld3(a.lx_out, j), lxo = ld3(a.lxo_out, j);
    for (uint32_t ep = rp; ep < re; ++ep) {
        const int i = (int)(a.ent[ep].x & END_MASK);
        if (a.rowp[i] & PIN_BIT) continue;  // a pinned vertex exerts no force adjoint
        const uint32_t e = a.rev[ep];
        const uint2 en = a.ent[e];
        const float k = a.kent ? a.kent[e] : list_k(P, en.x);
        V gx, gxo;
        double gk, gkd;
        spring_adj(ld3(a.x, i), ld3(a.xo, i), xj, xoj, k, __uint_as_float(en.y), P.kd, P.dt, ld3(a.G, i), gx, gxo, gk,
                   gkd);
        lx = lx - gx;
        lxo = lxo - gxo;
    }
    st3(a.lx_out, j, lx);
    st3(a.lxo_out, j, lxo);
}

}  // namespace

cudaError_t launch_step_f64(const double* x, const double* xo, double* xn, double* xon, double* nrm,
                            const uint32_t* rowp, const uint2* ent, const float* kent, const BvhView* bodies,
                            const float4* body_verts, const uint32_t* body_tris, const StepParams& p, int refv,
                            int collide, int n, int* err, unsigned* contacts, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_step_f64<<<(n + 255) / 256, 256, 0, s>>>(x, xo, xn, xon, nrm, rowp, ent, kent, bodies, body_verts, body_tris, p,
                                              refv, collide, n, err, contacts);
    return cudaGetLastError();
}

cudaError_t launch_widen(const float* src, double* dst, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_widen<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_narrow(const double* src, float* dst, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_narrow<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_step(const AdjArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    const unsigned g = (unsigned)((a.n + 255) / 256);
    k_adj_self<<<g, 256, 0, s>>>(a);
    k_adj_gather<<<g, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace visg
