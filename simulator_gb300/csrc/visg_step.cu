// visg_step.cu — the fused cloth step and the first-hit query.
//
// k_step is the reference's `verlet` kernel (src/verlet.cu:129-161) rebuilt for
// GB300: one thread per vertex, persistent CTAs walking a tile table (a tile is
// BLOCK consecutive vertices of one garment, so one launch covers any number of
// garments of uneven size), 32-byte interleaved state records (one float4 load per
// spring neighbour when spring damping is zero, two otherwise), springs of all
// lists merged into one sliced-ELL table of 8-byte entries (optionally staged per
// tile in shared memory by TMA bulk copies while the previous tile is computed)
// summed list by list with the list's stiffness uniform across the loop, the previous
// contact normal read only for vertices that had a contact, and the collision
// (collision_response_projection, verlet.cu:24-50) fused behind a warp vote on the
// body's root box.  Arithmetic follows the reference operation by operation with
// explicit round-to-nearest intrinsics:
//   v  = (x - xo) / dt
//   F  = g*m + v*damp;  F += sum_list (sum_entry spring);  F -= (n_prev.F) n_prev
//   spring = (-k (|d| - L0) + kd (dv.d)/|d|) * normalize(d),  d = x - x_j + FLT_EPSILON
//   x' = (x + x - xo) + (F/m*dt)*dt       (gamma == 1, verlet.cu:155)
//   x' = (x + gamma (x - xo)) + (F/m*dt)*dt  (damped Verlet)
//   first-hit leaf (cudaBRT.cu:239-285) -> plane test (primitive.cu:110-125)
//   -> x' += |dist| n, xo' = x', n_prev' = n; else n_prev' = 0
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>

#include "visg_internal.cuh"

namespace visg {

namespace {

constexpr float kFltEpsilon = 1.1920928955078125e-07f;  // FLT_EPSILON
constexpr int kStack = 32;  // > 30 = the depth bound of a radix tree over distinct 30-bit codes

__device__ __forceinline__ bool in_box(f3 p, float4 lo, float4 hi) {  // BBox::intersect, inclusive
    return (p.x >= lo.x && p.x <= hi.x) && (p.y >= lo.y && p.y <= hi.y) && (p.z >= lo.z && p.z <= hi.z);
}

// Upper bound of max_axis |a - b| (each difference rounded up).
__device__ __forceinline__ float disp_bound(f3 a, f3 b) {
    const float dx = __fsub_ru(fmaxf(a.x, b.x), fminf(a.x, b.x));
    const float dy = __fsub_ru(fmaxf(a.y, b.y), fminf(a.y, b.y));
    const float dz = __fsub_ru(fmaxf(a.z, b.z), fminf(a.z, b.z));
    return fmaxf(dx, fmaxf(dy, dz));
}

// Lower bounds (differences rounded down) of the L-infinity distance p can move
// before the closed-box test (BBox::intersect) changes its answer: outside the box,
// the largest per-axis gap; inside, the distance to the nearest face.
__device__ __forceinline__ float box_gap(f3 p, float4 lo, float4 hi) {
    return fmaxf(fmaxf(fmaxf(__fsub_rd(lo.x, p.x), __fsub_rd(p.x, hi.x)), fmaxf(__fsub_rd(lo.y, p.y), __fsub_rd(p.y, hi.y))),
                 fmaxf(__fsub_rd(lo.z, p.z), __fsub_rd(p.z, hi.z)));
}
__device__ __forceinline__ float box_inner(f3 p, float4 lo, float4 hi) {
    return fminf(fminf(fminf(__fsub_rd(p.x, lo.x), __fsub_rd(hi.x, p.x)), fminf(__fsub_rd(p.y, lo.y), __fsub_rd(hi.y, p.y))),
                 fminf(__fsub_rd(p.z, lo.z), __fsub_rd(hi.z, p.z)));
}

// D_BVH::intersect semantics: children tested pairwise; an overlapping leaf child is
// returned before any descent (A before B); both internal -> descend A, push B.
// The answer is therefore the first leaf, in a fixed order of the tree's leaves,
// whose box contains p (a node's box contains its children's).  A depth-first walk
// visits every internal node at most once, so `budget` (the number of internal
// nodes) bounds the loop even on a corrupted tree.
// With MARGIN, m receives a distance a point may move from p and keep the answer:
// every leaf before the answer lies under a box the walk rejected (min of their
// gaps), and the answer's own box must keep containing it (its inner distance).
template <bool MARGIN>
__device__ __forceinline__ int first_hit(const Node* __restrict__ nodes, int node, int budget, f3 p, int* err,
                                         float& m) {
    int stack[kStack];
    int sp = 0;
    while (true) {
        if (--budget < 0) {
            atomicOr(err, ERR_STACK);
            m = 0.0f;
            return -1;
        }
        const Node* nd = nodes + node;
        const float4 alo = __ldg(&nd->a_lo), ahi = __ldg(&nd->a_hi);
        const float4 blo = __ldg(&nd->b_lo), bhi = __ldg(&nd->b_hi);
        const int la = __float_as_int(alo.w), lb = __float_as_int(blo.w);
        const bool ol = in_box(p, alo, ahi), orr = in_box(p, blo, bhi);
        if (ol && la < 0) {
            if (MARGIN) m = fminf(m, box_inner(p, alo, ahi));
            return ~la;
        }
        if (MARGIN && !ol) m = fminf(m, box_gap(p, alo, ahi));
        if (orr && lb < 0) {
            if (MARGIN) m = fminf(m, box_inner(p, blo, bhi));
            return ~lb;
        }
        if (MARGIN && !orr) m = fminf(m, box_gap(p, blo, bhi));
        const bool tl = ol && la >= 0, tr = orr && lb >= 0;
        if (!tl && !tr) {
            if (sp == 0) return -1;
            node = stack[--sp];
        } else {
            node = tl ? la : lb;
            if (tl && tr) {
                if (sp == kStack) {
                    atomicOr(err, ERR_STACK);
                    m = 0.0f;
                    return -1;
                }
                stack[sp++] = lb;
            }
        }
    }
}

// The whole first-hit query of one body (root box, single leaf, walk) with its margin.
__device__ __forceinline__ int query_margin(const BvhView& bv, f3 p, int* err, float& m) {
    const int nl = bv.root->n_leaves;
    const float4 lo = bv.root->top_lo, hi = bv.root->top_hi;
    if (!in_box(p, lo, hi)) {
        m = fminf(m, box_gap(p, lo, hi));
        return -1;
    }
    if (nl == 1) {
        m = fminf(m, box_inner(p, lo, hi));
        return 0;
    }
    return first_hit<true>(bv.nodes, bv.root->root, nl, p, err, m);
}

__device__ __forceinline__ int query_leaf(const BvhView& bv, int n_leaves, int root, float4 top_lo, float4 top_hi,
                                          f3 p, int* err) {
    if (n_leaves <= 0 || !in_box(p, top_lo, top_hi)) return -1;
    if (n_leaves == 1) return 0;
    float m = 0.0f;
    return first_hit<false>(bv.nodes, root, n_leaves, p, err, m);
}

// Force of one spring on the vertex at x moving with velocity vel (verlet.cu:64-84):
//   c = -k (|d| - L0) + kd (dv.d) / |d|,  force = c * normalize(d),  d = x - x_j + FLT_EPSILON
// t0/t1 is the neighbour's record: position and velocity (p2 - p2_old) / dt, stored
// once per step by the neighbour's own thread with the same IEEE division; nk = -k.
// FAST drops the damping term, for spring damping exactly +0: see row_forces.
// With drec the neighbour's record holds D = p2 - p2_old; its velocity is D / dt.
template <bool FAST>
__device__ __forceinline__ f3 spring_force(f3 x, f3 vel, float4 t0, float4 t1, float nk, float rest, float kd,
                                           f3 eps3, bool drec, float dt) {
    const f3 dP = add(sub(x, mk3(t0.x, t0.y, t0.z)), eps3);
    const float dist = __fsqrt_rn(dot(dP, dP));
    float c = __fmul_rn(nk, __fsub_rn(dist, rest));
    if (!FAST) {
        f3 v2 = mk3(t0.w, t1.x, t1.y);
        if (drec) v2 = divs(v2, dt);
        const f3 dV = sub(vel, v2);
        c = __fadd_rn(c, __fmul_rn(kd, __fdiv_rn(dot(dV, dP), dist)));
    }
    return mul(c, mul(dP, __frcp_rn(dist)));  // normalize(dP) = dP * (1 / |dP|)
}

// Two springs of one vertex at once, spring damping exactly +0 (spring_force<true>
// on each spring, operation for operation).  The x and y components of a spring's
// vectors travel as one packed pair (a record's x, y are adjacent words), z alone;
// the two springs' scalar chains (|dP|^2, the square root and its reciprocal, the
// rest-length term) travel as one pair.  Every packed operation rounds each lane as
// the scalar intrinsic would, and sqrt_rcp_pair returns __fsqrt_rn / __frcp_rn's
// bits, so each force is bit-identical to the scalar form in fewer instructions
// (sm_100+ f32x2 arithmetic).
__device__ __forceinline__ void spring_pair(fp2 xxy, float xz, float4 ta, float4 tb, fp2 nk, fp2 rest, fp2 eps2,
                                            float eps, fp2& f_xy_a, float& fz_a, fp2& f_xy_b, float& fz_b) {
    const fp2 da = add2(sub2(xxy, pk2(ta.x, ta.y)), eps2), db = add2(sub2(xxy, pk2(tb.x, tb.y)), eps2);
    const float dza = __fadd_rn(__fsub_rn(xz, ta.z), eps), dzb = __fadd_rn(__fsub_rn(xz, tb.z), eps);
    const fp2 qa = mul2(da, da), qb = mul2(db, db);
    const fp2 s = pk2(__fadd_rn(__fadd_rn(lo2(qa), hi2(qa)), __fmul_rn(dza, dza)),
                      __fadd_rn(__fadd_rn(lo2(qb), hi2(qb)), __fmul_rn(dzb, dzb)));  // dot(dP, dP)
    fp2 dist, inv;
    sqrt_rcp_pair(s, dist, inv);
    const fp2 c = mul2(nk, sub2(dist, rest));  // -k (|dP| - L0)
    const float ca = lo2(c), cb = hi2(c), ia = lo2(inv), ib = hi2(inv);
    f_xy_a = pk2(__fmul_rn(ca, __fmul_rn(lo2(da), ia)), __fmul_rn(ca, __fmul_rn(hi2(da), ia)));
    fz_a = __fmul_rn(ca, __fmul_rn(dza, ia));
    f_xy_b = pk2(__fmul_rn(cb, __fmul_rn(lo2(db), ib)), __fmul_rn(cb, __fmul_rn(hi2(db), ib)));
    fz_b = __fmul_rn(cb, __fmul_rn(dzb, ib));
}

// One 16-byte load that the compiler may not merge with an earlier load of the same
// address (a value read again later instead of being held in registers meanwhile).
__device__ __forceinline__ float4 ld_once(const float4* p) {
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}

// Contact data a vertex will read after its spring sum (its cached leaf, its stored
// normal), prefetched when the vertex starts: 0 = not prefetched, 1 = into L1, 2 = L2.
// Those reads otherwise start a dependent DRAM round trip at the end of every warp
// with a contact in it; prefetched into L2 the step kernel takes 0.272 ms against
// 0.278 over the 256-garment draped batch (into L1: the same).
constexpr int kPrefetchContact = 2;
__device__ __forceinline__ void prefetch_contact(const void* p) {
    if (kPrefetchContact == 1) asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
    if (kPrefetchContact == 2) asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Vertex records are read through the read-only path (about half the neighbour
// reads hit L1: rows of a grid share most neighbours).
struct GlobalRecords {
    const float4* __restrict__ p;
    __device__ __forceinline__ float4 r0(int j) const { return __ldg(p + 2 * j); }
    __device__ __forceinline__ float4 r1(int j) const { return __ldg(p + 2 * j + 1); }
};

// A row's sliced-ELL entries (entry e at p[32 e]): in global memory, or in the tile's
// block that a TMA bulk copy staged in shared memory.
template <bool SMEM>
struct Entries {
    const uint2* p;
    __device__ __forceinline__ uint2 operator[](int e) const { return SMEM ? p[32 * e] : __ldg(p + 32 * e); }
};

// Sum of springs [e, end) of one list of a sliced-ELL row (ep/kp at the row's entry
// 0, entries 32 apart), in CSR order, two at a time (independent chains).
template <bool FAST, class Rec, class Ent>
__device__ __forceinline__ f3 list_sum(const Rec& rec, const Ent& ep, const float* __restrict__ kp, int e,
                                       const int end, const float nk, const bool perk, f3 x, f3 vel, float kd,
                                       f3 eps3, bool drec, float dt) {
    f3 acc = mk3(0.0f, 0.0f, 0.0f);
    if (FAST) {  // two springs per packed evaluation; the sum stays in CSR order
        const fp2 xxy = pk2(x.x, x.y), eps2 = splat2(eps3.x), nk2 = splat2(nk);
        fp2 axy = pk2(0.0f, 0.0f);
        float az = 0.0f;
        for (; e + 1 < end; e += 2) {
            const uint2 ea = ep[e], eb = ep[e + 1];
            const int ja = (int)(ea.x & END_MASK), jb = (int)(eb.x & END_MASK);
            const float4 a0 = rec.r0(ja), b0 = rec.r0(jb);
            const fp2 k2 = perk ? pk2(-__ldg(kp + 32 * e), -__ldg(kp + 32 * (e + 1))) : nk2;
            fp2 fa, fb;
            float fza, fzb;
            spring_pair(xxy, x.z, a0, b0, k2, pk2(__uint_as_float(ea.y), __uint_as_float(eb.y)), eps2, eps3.x, fa, fza,
                        fb, fzb);
            axy = add2(add2(axy, fa), fb);
            az = __fadd_rn(__fadd_rn(az, fza), fzb);
        }
        acc = mk3(lo2(axy), hi2(axy), az);
        if (e < end) {
            const uint2 ea = ep[e];
            const float4 a0 = rec.r0((int)(ea.x & END_MASK));
            const float ka = perk ? -__ldg(kp + 32 * e) : nk;
            acc = add(acc, spring_force<true>(x, vel, a0, a0, ka, __uint_as_float(ea.y), kd, eps3, drec, dt));
        }
        return acc;
    }
    for (; e + 1 < end; e += 2) {
        const uint2 ea = ep[e], eb = ep[e + 1];
        const int ja = (int)(ea.x & END_MASK), jb = (int)(eb.x & END_MASK);
        const float4 a0 = rec.r0(ja), b0 = rec.r0(jb);
        const float4 a1 = FAST ? a0 : rec.r1(ja), b1 = FAST ? b0 : rec.r1(jb);
        const float ka = perk ? -__ldg(kp + 32 * e) : nk;
        const float kb = perk ? -__ldg(kp + 32 * (e + 1)) : nk;
        const f3 fa = spring_force<FAST>(x, vel, a0, a1, ka, __uint_as_float(ea.y), kd, eps3, drec, dt);
        const f3 fb = spring_force<FAST>(x, vel, b0, b1, kb, __uint_as_float(eb.y), kd, eps3, drec, dt);
        acc = add(add(acc, fa), fb);
    }
    if (e < end) {
        const uint2 ea = ep[e];
        const int ja = (int)(ea.x & END_MASK);
        const float4 a0 = rec.r0(ja);
        const float4 a1 = FAST ? a0 : rec.r1(ja);
        const float ka = perk ? -__ldg(kp + 32 * e) : nk;
        acc = add(acc, spring_force<FAST>(x, vel, a0, a1, ka, __uint_as_float(ea.y), kd, eps3, drec, dt));
    }
    return acc;
}

// F + the spring forces of one vertex, list by list as the reference does
// (force += list sum, verlet.cu:148-149); cnt holds the row's per-list counts.
template <bool FAST, class Rec, class Ent>
__device__ __forceinline__ f3 row_forces(const Rec& rec, const Ent& ep, const float* __restrict__ kp, uint2 cnt,
                                         f3 x, f3 vel, f3 F, const StepParams& P, bool perk, f3 eps3) {
    int e = 0;
#pragma unroll
    for (int l = 0; l < VISG_MAX_LISTS; ++l) {
        if (l < P.n_lists) {
            const int n = (int)(((l < 2 ? cnt.x : cnt.y) >> (16 * (l & 1))) & (l == 3 ? 0x7fffu : 0xffffu));
            F = add(F, list_sum<FAST>(rec, ep, kp, e, e + n, -P.list_k[l], perk, x, vel, P.kd, eps3, P.drec != 0,
                                      P.dt));
            e += n;
        }
    }
    return F;
}

// |x| < 1e15 and |v| < 1e15 in every component (false for NaN): while every record
// satisfies this, RN(dv.d / |d|) is finite for every spring (|dv.d| < 3 (2e15)^2,
// |d| within a factor ~2 of max |d_i| unless it underflows to 0).
__device__ __forceinline__ bool tame(f3 x, f3 v) {
    const float m = 1e15f;
    return fabsf(x.x) < m && fabsf(x.y) < m && fabsf(x.z) < m && fabsf(v.x) < m && fabsf(v.y) < m && fabsf(v.z) < m;
}
// the same for a record that carries D = x - x_old (dmax = 0.5e15 dt, so |D / dt| < 1e15)
__device__ __forceinline__ bool tame_d(f3 x, f3 d, float dmax) {
    const float m = 1e15f;
    return fabsf(x.x) < m && fabsf(x.y) < m && fabsf(x.z) < m && fabsf(d.x) < dmax && fabsf(d.y) < dmax &&
           fabsf(d.z) < dmax;
}

// One thread's vertex of tile td = {garment, first vertex, end vertex, first slice}.
// State record of vertex i in buffer b: [x.xyz, v.x] [v.y, v.z, flags, 0] with
// v = (x - x_old) / dt.  x_old is x itself when FLAG_XO_IS_X is set (after a
// contact, a pin or update_vertex) and otherwise the previous step's x, which is
// still in the other buffer: the step reads it there before overwriting it.
template <bool COLL, bool KD0, bool SPLIT, bool SMEM_ENT>
__device__ __forceinline__ void vertex_step(const StepArgs& a, const int4 td, const uint2* ebase, const uint32_t e0,
                                            const int refv, const int check, const int perk, const bool wild,
                                            float& my_disp, uint32_t& my_bad) {
    const GlobalRecords rec{a.state_in};
    const StepParams& P = a.p;
    const f3 grav = mk3(P.gx, P.gy, P.gz);
    const f3 eps3 = mk3(kFltEpsilon, kFltEpsilon, kFltEpsilon);
    const int i = td.y + (int)threadIdx.x;
    const bool active = i < td.z;
    const int ii = active ? i : td.y;
    const float4 s0 = rec.r0(ii);
    const f3 x = mk3(s0.x, s0.y, s0.z);
    const uint2 cnt = __ldg(&a.vcount[ii]);
    const bool pinned = (cnt.y & PIN_BIT) != 0u;
    if (COLL && kPrefetchContact) {
        // the record's flags word (the sector s0 came in): start the loads that a cached
        // contact answer and a stored normal need after the spring sum
        const uint32_t fl0 = __float_as_uint(__ldg(reinterpret_cast<const float*>(a.state_in + 2 * ii + 1) + 2));
        if (fl0 & FLAG_LEAF_CACHED)
            prefetch_contact(a.bodies[td.x & TILE_GARMENT].leaves + 2 * (fl0 >> LEAF_SHIFT));
        if (fl0 & FLAG_HAS_NORMAL) prefetch_contact(a.normal + ii);
    }
    f3 xn = x, xon = x, nn = mk3(0.0f, 0.0f, 0.0f);
    bool has_n = false;
    uint32_t flags = 0u;
    float margin = 0.0f;
    if (active && !pinned) {
        const int lane = (int)(threadIdx.x & 31u);
        const uint32_t sb = __ldg(&a.slice_off[td.w + (int)(threadIdx.x >> 5)]) + (uint32_t)lane;  // row entry 0
        // The zero-damping sum needs only positions: there the rest of the record
        // (v or D, flags, the query cache's margin) is read after the sum, not held in
        // registers across it.  With drec and force damping exactly +0 the term v * +0
        // is a signed zero for every tame v, and g m + (+-0) only differs in the sign
        // of a zero component, which the first list's sum (never -0) erases.
        const bool pos_only = KD0 && P.drec && __float_as_uint(P.damp) == 0u && !wild;
        f3 vel = mk3(0.0f, 0.0f, 0.0f);
        f3 F0 = mul(grav, P.mass);
        if (!pos_only) {
            const float4 s1 = rec.r1(ii);
            const f3 rv = mk3(s0.w, s1.x, s1.y);  // v, or D = x - x_old with drec
            vel = P.drec ? divs(rv, P.dt) : rv;
            if (!P.drec || __float_as_uint(P.damp) != 0u || wild) F0 = add(F0, mul(vel, P.damp));
        }
        const Entries<SMEM_ENT> ep{ebase + (sb - e0)};
        const float* kp = perk ? a.sellk + sb : nullptr;
        f3 F;
        if (KD0) {
            // Spring damping is +0: the reference adds +0 * RN(dv.d / |d|) to every c.
            // Without it c differs at most in the sign of a zero, which changes no sum
            // (a zero force adds nothing to sums that start at +0, which never become -0),
            // as long as RN(dv.d / |d|) is finite (guaranteed while every record is tame;
            // the wild flag says when one was not) or c is not finite (then F is not
            // finite either: such rows are recomputed with the damping term).
            F = row_forces<true>(rec, ep, kp, cnt, x, vel, F0, P, perk != 0, eps3);
        } else {
            F = row_forces<false>(rec, ep, kp, cnt, x, vel, F0, P, perk != 0, eps3);
        }
        // the record again (a second read of a line this thread has just read)
        const float4 r0 = ld_once(a.state_in + 2 * ii), r1 = ld_once(a.state_in + 2 * ii + 1);
        const f3 rv = mk3(r0.w, r1.x, r1.y);  // v, or D = x - x_old with drec
        flags = __float_as_uint(r1.z);
        margin = r1.w;
        if (KD0 && (wild || !(isfinite(F.x) && isfinite(F.y) && isfinite(F.z)))) {
            vel = P.drec ? divs(rv, P.dt) : rv;
            F = row_forces<false>(rec, ep, kp, cnt, x, vel, F0, P, perk != 0, eps3);
        }
        // x - x_old: from the record (drec), else from x_old in the other buffer
        f3 xo = x, d = rv;
        if (!P.drec) {
            if (!(flags & FLAG_XO_IS_X)) xo = xyz(a.state_out[2 * ii]);
            d = sub(x, xo);
        }
        f3 np = mk3(0.0f, 0.0f, 0.0f);
        if (flags & FLAG_HAS_NORMAL) np = xyz(a.normal[ii]);
        F = sub(F, mul(dot(np, F), np));  // inelastic response (verlet.cu:151-152)
        const f3 adt = mul(mul(divs(F, P.mass), P.dt), P.dt);
        if (refv) xn = add(sub(add(x, x), xo), adt);  // never with drec
        else xn = add(add(x, mul(P.gamma, d)), adt);
        xon = x;
    }
    // Query cache.  s1.w holds a margin: while the vertex stays within that L-infinity
    // distance of the point its last first-hit query was answered at, the query's
    // answer is unchanged (first_hit's margin) and is reused: no leaf, or the leaf in
    // the flags word (FLAG_LEAF_CACHED), whose plane test is redone at the new position.
    // The margin shrinks by every displacement since (rounded up); 0 = no cache.
    float skin = 0.0f;
    uint32_t leaf_bits = 0u;  // the cached leaf, in the flags word's place (0: no leaf cached)
    if (COLL) {
        const int g = td.x & TILE_GARMENT;
        const bool body = (td.x & TILE_BODY) != 0;  // the garment has a body (its tree has leaves)
        bool query = false;
        int leaf = -1;
        if (body && active && !pinned) {
            const float rem = P.margin ? __fsub_rd(margin, disp_bound(xn, x)) : 0.0f;
            if (rem > 0.0f) {
                skin = rem;
                if (flags & FLAG_LEAF_CACHED) {
                    leaf = (int)(flags >> LEAF_SHIFT);
                    leaf_bits = (flags & ~7u) | FLAG_LEAF_CACHED;
                }
            } else {
                query = true;
            }
        }
        if (SPLIT) {
            // queue the queries (one atomic per warp); k_collide answers them with fully
            // populated warps and stores their margins
            const unsigned m = __ballot_sync(0xffffffffu, query);
            if (m) {
                const int lane = (int)(threadIdx.x & 31u), leader = __ffs(m) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(a.cand_count, (uint32_t)__popc(m));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (query) a.cand[base + __popc(m & ((1u << lane) - 1u))] = make_int2(i, g);
            }
        } else if (__any_sync(0xffffffffu, query) && query) {
            float m = __int_as_float(0x7f800000);  // +inf
            leaf = query_margin(a.bodies[g], xn, a.err, m);
            if (P.margin) {
                skin = m;
                if (leaf >= 0 && leaf < kLeafCacheMax) leaf_bits = ((uint32_t)leaf << LEAF_SHIFT) | FLAG_LEAF_CACHED;
            }
        }
        if (leaf >= 0) {  // plane test of the first-hit leaf (primitive.cu:110-125)
            const float4* const leaves = a.bodies[g].leaves;
            const float4 L0 = __ldg(&leaves[2 * leaf]);
            const float4 L1 = __ldg(&leaves[2 * leaf + 1]);
            const f3 n = mk3(L0.w, L1.x, L1.y);
            const float d = dot(sub(xn, mk3(L0.x, L0.y, L0.z)), n);
            if (!(d > 0.0f)) {
                const f3 xp = add(xn, mul(__fmul_rn(1.0f, fabsf(d)), n));
                skin = __fsub_rd(skin, disp_bound(xp, xn));
                xn = xp;
                xon = xn;
                nn = n;
                has_n = true;
            }
        }
    }
    bool untamed = false;
    if (active) {
        const bool xo_is_x = pinned || has_n;
        const f3 dn = sub(xn, xon);
        const f3 vn = P.drec ? dn : divs(dn, P.dt);  // what the record carries
        untamed = P.drec ? !tame_d(xn, dn, P.dmax) : !tame(xn, vn);
        const uint32_t fl = (has_n ? FLAG_HAS_NORMAL : 0u) | (xo_is_x ? FLAG_XO_IS_X : 0u) |
                            (skin > 0.0f ? leaf_bits : 0u);
        a.state_out[2 * i] = make_float4(xn.x, xn.y, xn.z, vn.x);
        a.state_out[2 * i + 1] = make_float4(vn.y, vn.z, __uint_as_float(fl), skin > 0.0f ? skin : 0.0f);
        if (has_n) a.normal[i] = make_float4(nn.x, nn.y, nn.z, 0.0f);
        if (check) {
            const float dd = fmaxf(fabsf(__fsub_rn(xn.x, x.x)),
                                   fmaxf(fabsf(__fsub_rn(xn.y, x.y)), fabsf(__fsub_rn(xn.z, x.z))));
            const f3 vc = P.drec ? divs(dn, P.dt) : vn;
            if (!isfinite(xn.x) || !isfinite(xn.y) || !isfinite(xn.z) || !isfinite(vc.x) || !isfinite(vc.y) ||
                !isfinite(vc.z))
                ++my_bad;
            else
                my_disp = fmaxf(my_disp, dd);
        }
    }
    if (__any_sync(0xffffffffu, untamed) && (threadIdx.x & 31u) == 0u) atomicOr(a.wild, 1u);
}

// ---- TMA bulk copies into shared memory, completed on an mbarrier ----------------------
constexpr int kBarBytes = 128;                 // two 8-byte mbarriers, padded
constexpr uint64_t kWaitNs = 1000000000ull;    // a stage that has not landed after 1 s is an error

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// one arrival that also announces `bytes` of transactions, then the copy that completes them
__device__ __forceinline__ void bulk_stage(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0u;
}

// bounded wait for the phase of the given parity to complete
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_test(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_test(bar, parity))
        if (global_ns() - t0 > kWaitNs) return false;
    return true;
}

// the stager: stage the sliced-ELL block of `tile` at shared address dst, completing
// the buffer's `full` phase when it lands; a tile without a staged block completes
// the phase at once (every tile takes one phase, so no warp runs ahead of the ring)
__device__ __forceinline__ void stage_entries(const StepArgs& a, int tile, uint32_t dst, uint32_t full) {
    const int2 tw = __ldg(&a.twin[tile]);
    if (tw.y > 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the readers' loads come first
        bulk_stage(dst, a.sell + (uint32_t)tw.x, (uint32_t)tw.y * 8u, full);
    } else {
        mbar_arrive(full);
    }
}

// The fused step: persistent CTAs walk the tile table.  With STAGED, one thread (the
// stager) copies the next tile's block of sliced-ELL entries (the tile's slices are
// contiguous: one TMA bulk copy) into the other shared-memory buffer while the warps
// compute the current tile, so each spring's chain starts with a shared-memory load;
// tiles whose block exceeds the buffer read their entries from global memory.  No CTA
// barrier per tile: warps report a finished buffer on its `empty` mbarrier and only
// the stager waits for it before refilling.  The stager of iteration `it` is lane 0 of
// warp it % (BLOCK / 32), so the wait for the slowest warp and the copy's issue
// latency fall on each warp once per BLOCK / 32 tiles.  With thread 0 as the only
// stager they fell on warp 0 every tile, and warp 0 paced the CTA: the other warps
// ran up to a tile ahead and then waited on `full`.  Waits are bounded: one that
// gives up after kWaitNs sets ERR_TIMEOUT, the iteration's stager waits (again
// bounded) for the copies in flight, and the warp exits; warps left waiting on a
// copy that is never issued give up the same way.
template <int BLOCK, bool COLL, bool KD0, bool SPLIT, bool STAGED>
__global__ void __launch_bounds__(BLOCK) k_step(const StepArgs a, const int refv, const int check, const int perk) {
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    float my_disp = 0.0f;
    uint32_t my_bad = 0;
    const bool wild = *reinterpret_cast<const volatile uint32_t*>(a.wild) != 0u;
    if (!STAGED) {
        for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x)
            vertex_step<COLL, KD0, SPLIT, false>(a, __ldg(&a.tiles[tile]), a.sell, 0u, refv, check, perk, wild,
                                                 my_disp, my_bad);
    } else {
        // two-buffer ring: full[b] completes when buffer b holds its tile's block,
        // empty[b] when every warp is done reading it
        const uint32_t full = smem_addr(dyn_smem), empty = full + 16u;
        const uint32_t buf0 = full + kBarBytes;
        const uint2* sbuf = reinterpret_cast<const uint2*>(dyn_smem + kBarBytes);
        const uint32_t bbytes = (uint32_t)a.win_cap * 8u;
        const int lane = (int)(threadIdx.x & 31u);
        if (threadIdx.x == 0) {
            mbar_init(full, 1u);
            mbar_init(full + 8u, 1u);
            mbar_init(empty, BLOCK / 32);
            mbar_init(empty + 8u, BLOCK / 32);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (threadIdx.x == 0 && (int)blockIdx.x < a.n_tiles) stage_entries(a, blockIdx.x, buf0, full);
        int it = 0;
        for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++it) {
            const int b = it & 1;
            const uint32_t par = (uint32_t)(it >> 1) & 1u;  // phase parity of this iteration's buffer
            const int nxt = tile + (int)gridDim.x;
            const uint32_t stager = (uint32_t)(it % (BLOCK / 32)) * 32u;
            bool pok = true;
            if (threadIdx.x == stager && nxt < a.n_tiles) {
                // the other buffer was read in iteration it - 1: wait for every warp to finish it
                if (it >= 1) pok = mbar_wait(empty + 8u * (b ^ 1), (uint32_t)((it - 1) >> 1) & 1u);
                if (pok) stage_entries(a, nxt, buf0 + (uint32_t)(b ^ 1) * bbytes, full + 8u * (b ^ 1));
            }
            const bool landed = mbar_wait(full + 8u * b, par);
            if (!__all_sync(0xffffffffu, landed && pok)) {
                // a wait gave up: record it; the stager lets the copies in flight land
                if (lane == 0) atomicOr(a.err, ERR_TIMEOUT);
                if (threadIdx.x == stager) {
                    mbar_wait(full + 8u * b, par);
                    if (pok && nxt < a.n_tiles) mbar_wait(full + 8u * (b ^ 1), (uint32_t)((it + 1) >> 1) & 1u);
                }
                return;
            }
            const int4 td = __ldg(&a.tiles[tile]);
            const int2 tw = __ldg(&a.twin[tile]);
            if (tw.y > 0)
                vertex_step<COLL, KD0, SPLIT, true>(a, td, sbuf + (size_t)b * a.win_cap, (uint32_t)tw.x, refv, check,
                                                    perk, wild, my_disp, my_bad);
            else
                vertex_step<COLL, KD0, SPLIT, false>(a, td, a.sell, 0u, refv, check, perk, wild, my_disp, my_bad);
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + 8u * b);
        }
    }
    if (check) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            my_disp = fmaxf(my_disp, __shfl_xor_sync(0xffffffffu, my_disp, o));
            my_bad += __shfl_xor_sync(0xffffffffu, my_bad, o);
        }
        if ((threadIdx.x & 31) == 0) {
            if (my_disp > 0.0f) atomicMax(&a.check[0], __float_as_uint(my_disp));
            if (my_bad) atomicAdd(&a.check[1], my_bad);
        }
    }
}

// Split collision (collision_response_projection, verlet.cu:24-50): the queued
// first-hit queries.  The integrate pass has already written each record as if it
// had no contact (flags without a cache, margin 0); a projected vertex gets
// x' += |dist| n, x_old' = x', v' = 0 and its normal; every answered query stores its
// margin (and leaf) for the query cache.
constexpr int COLLIDE_BLOCK = 256;
__global__ void __launch_bounds__(COLLIDE_BLOCK) k_collide(const StepArgs a) {
    const uint32_t n = *a.cand_count;
    const float dt = a.p.dt;
    for (uint32_t k = blockIdx.x * COLLIDE_BLOCK + threadIdx.x; k < n; k += gridDim.x * COLLIDE_BLOCK) {
        const int2 c = a.cand[k];
        const BvhView bv = a.bodies[c.y];
        float4 s0 = a.state_out[2 * c.x], s1 = a.state_out[2 * c.x + 1];
        f3 xn = mk3(s0.x, s0.y, s0.z);
        float m = __int_as_float(0x7f800000);  // +inf
        const int leaf = query_margin(bv, xn, a.err, m);
        uint32_t fl = __float_as_uint(s1.z);
        float skin = a.p.margin ? m : 0.0f;
        if (leaf >= 0) {
            if (a.p.margin && leaf < kLeafCacheMax) fl |= ((uint32_t)leaf << LEAF_SHIFT) | FLAG_LEAF_CACHED;
            const float4 L0 = __ldg(&bv.leaves[2 * leaf]);
            const float4 L1 = __ldg(&bv.leaves[2 * leaf + 1]);
            const f3 nrm = mk3(L0.w, L1.x, L1.y);
            const float d = dot(sub(xn, mk3(L0.x, L0.y, L0.z)), nrm);
            if (!(d > 0.0f)) {
                const f3 xp = add(xn, mul(__fmul_rn(1.0f, fabsf(d)), nrm));
                skin = __fsub_rd(skin, disp_bound(xp, xn));
                xn = xp;
                const f3 vn = divs(sub(xn, xn), dt);
                s0 = make_float4(xn.x, xn.y, xn.z, vn.x);
                s1.x = vn.y;
                s1.y = vn.z;
                fl |= FLAG_HAS_NORMAL | FLAG_XO_IS_X;
                a.state_out[2 * c.x] = s0;
                a.normal[c.x] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
                if (!tame(xn, vn)) atomicOr(a.wild, 1u);
            }
        }
        if (!(skin > 0.0f)) {
            skin = 0.0f;
            fl &= 7u & ~FLAG_LEAF_CACHED;
        }
        a.state_out[2 * c.x + 1] = make_float4(s1.x, s1.y, __uint_as_float(fl), skin);
    }
}

int g_collide_grid = 0;

// the step kernel instance of a variant
template <int BLOCK, bool KD0, bool STAGED>
using StepKernel = void (*)(const StepArgs, const int, const int, const int);

template <int BLOCK, bool KD0, bool STAGED>
StepKernel<BLOCK, KD0, STAGED> step_kernel(bool coll, bool split) {
    if (coll && split) return k_step<BLOCK, true, KD0, true, STAGED>;
    if (coll) return k_step<BLOCK, true, KD0, false, STAGED>;
    return k_step<BLOCK, false, KD0, false, STAGED>;
}

// largest dynamic shared memory each kernel instance has been opened up to (per device)
std::mutex g_smem_mu;
std::map<std::pair<int, const void*>, int> g_smem_set;

cudaError_t allow_smem(const void* fn, int bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_smem_mu);
    int& cur = g_smem_set[{dev, fn}];
    if (cur >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

// events recorded right before and after each step-kernel launch of this thread
// (kernel timing; null = none)
thread_local cudaEvent_t t_before_step = nullptr, t_after_step = nullptr;

template <int BLOCK, bool KD0, bool STAGED>
cudaError_t launch_kd(const StepArgs& a, bool coll, bool split, int refv, int check, int perk, int grid, int smem,
                      cudaStream_t s) {
    const auto fn = step_kernel<BLOCK, KD0, STAGED>(coll, split);
    cudaError_t e = allow_smem((const void*)fn, smem);
    if (e != cudaSuccess) return e;
    if (coll && split) {
        e = cudaMemsetAsync(a.cand_count, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
    }
    if (t_before_step) cudaEventRecord(t_before_step, s);
    fn<<<grid, BLOCK, smem, s>>>(a, refv, check, perk);
    if (t_after_step) cudaEventRecord(t_after_step, s);
    if (coll && split) {
        if (g_collide_grid == 0) {
            int dev = 0, sms = 0, occ = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_collide, COLLIDE_BLOCK, 0);
            // two CTAs per SM walk the queue (grid-stride): threads for the usual queue
            // without idle CTAs competing for slots with the other group's step
            g_collide_grid = sms * (occ >= 2 ? 2 : 1);
        }
        k_collide<<<g_collide_grid, COLLIDE_BLOCK, 0, s>>>(a);
    }
    return cudaGetLastError();
}

template <int BLOCK>
cudaError_t launch_block(const StepArgs& a, int variant, int grid, cudaStream_t s) {
    const int refv = (variant & SV_REFV) ? 1 : 0;
    const int check = (variant & SV_CHECK) ? 1 : 0;
    const int perk = (variant & SV_PERK) ? 1 : 0;
    const bool coll = (variant & SV_COLLIDE) != 0, split = (variant & SV_SPLIT) != 0;
    const int smem = step_smem_bytes(variant, a.win_cap);
    if (variant & SV_STAGED) {
        if (variant & SV_KD0) return launch_kd<BLOCK, true, true>(a, coll, split, refv, check, perk, grid, smem, s);
        return launch_kd<BLOCK, false, true>(a, coll, split, refv, check, perk, grid, smem, s);
    }
    if (variant & SV_KD0) return launch_kd<BLOCK, true, false>(a, coll, split, refv, check, perk, grid, 0, s);
    return launch_kd<BLOCK, false, false>(a, coll, split, refv, check, perk, grid, 0, s);
}

template <int BLOCK, bool KD0, bool STAGED>
int occupancy_kd(bool coll, bool split, int smem) {
    const auto fn = step_kernel<BLOCK, KD0, STAGED>(coll, split);
    if (allow_smem((const void*)fn, smem) != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, BLOCK, smem) != cudaSuccess) return 0;
    return n;
}

template <int BLOCK>
int occupancy_block(int variant, int win_cap) {
    const bool coll = (variant & SV_COLLIDE) != 0, split = (variant & SV_SPLIT) != 0;
    const int smem = step_smem_bytes(variant, win_cap);
    if (variant & SV_STAGED)
        return (variant & SV_KD0) ? occupancy_kd<BLOCK, true, true>(coll, split, smem)
                                  : occupancy_kd<BLOCK, false, true>(coll, split, smem);
    return (variant & SV_KD0) ? occupancy_kd<BLOCK, true, false>(coll, split, 0)
                              : occupancy_kd<BLOCK, false, false>(coll, split, 0);
}

__global__ void k_query(BvhView bv, const float* __restrict__ pts, int n, int* leaf, int* inside, float* dist,
                        float* normal, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 p = mk3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    const int nl = bv.root->n_leaves;
    const int lf = query_leaf(bv, nl, bv.root->root, bv.root->top_lo, bv.root->top_hi, p, err);
    float d = 0.0f;
    f3 nn = mk3(0.0f, 0.0f, 0.0f);
    int in = 0;
    if (lf >= 0) {
        const float4 L0 = bv.leaves[2 * lf], L1 = bv.leaves[2 * lf + 1];
        nn = mk3(L0.w, L1.x, L1.y);
        d = dot(sub(p, mk3(L0.x, L0.y, L0.z)), nn);
        in = !(d > 0.0f);
    }
    if (leaf) leaf[i] = lf;
    if (inside) inside[i] = in;
    if (dist) dist[i] = d;
    if (normal) {
        normal[3 * i] = nn.x;
        normal[3 * i + 1] = nn.y;
        normal[3 * i + 2] = nn.z;
    }
}

__global__ void k_unpack_positions(const float4* __restrict__ st, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s0 = st[2 * i];
    out[3 * i] = s0.x;
    out[3 * i + 1] = s0.y;
    out[3 * i + 2] = s0.z;
}

__global__ void k_unpack_state(const float4* __restrict__ st, const float4* __restrict__ other,
                               const float4* __restrict__ nr, int64_t n, float* x, float* xo, float* nrm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s0 = st[2 * i], s1 = st[2 * i + 1];
    const uint32_t fl = __float_as_uint(s1.z);
    if (x) { x[3 * i] = s0.x; x[3 * i + 1] = s0.y; x[3 * i + 2] = s0.z; }
    if (xo) {
        const float4 o = (fl & FLAG_XO_IS_X) ? s0 : other[2 * i];
        xo[3 * i] = o.x; xo[3 * i + 1] = o.y; xo[3 * i + 2] = o.z;
    }
    if (nrm) {
        const float4 v = (fl & FLAG_HAS_NORMAL) ? nr[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        nrm[3 * i] = v.x; nrm[3 * i + 1] = v.y; nrm[3 * i + 2] = v.z;
    }
}

// x == nullptr keeps x, etc.  x_old is written into the other buffer and v is
// recomputed as (x - x_old) / dt; a vertex has a stored normal iff it is non-zero.
__global__ void k_pack_state(float4* st, float4* other, float4* nr, int64_t n, const float* x, const float* xo,
                             const float* nrm, float dt, int drec, float dmax, uint32_t* wild) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 s0 = st[2 * i], s1 = st[2 * i + 1];
    uint32_t fl = __float_as_uint(s1.z) & (FLAG_HAS_NORMAL | FLAG_XO_IS_X);  // no cached answer
    const f3 x0 = mk3(s0.x, s0.y, s0.z);
    const f3 xo0 = (fl & FLAG_XO_IS_X) ? x0 : xyz(other[2 * i]);
    const f3 xv = x ? mk3(x[3 * i], x[3 * i + 1], x[3 * i + 2]) : x0;
    const f3 xov = xo ? mk3(xo[3 * i], xo[3 * i + 1], xo[3 * i + 2]) : xo0;
    const f3 v = drec ? sub(xv, xov) : divs(sub(xv, xov), dt);  // what the record carries
    if (nrm) {
        const float a = nrm[3 * i], b = nrm[3 * i + 1], c = nrm[3 * i + 2];
        const bool h = a != 0.0f || b != 0.0f || c != 0.0f;
        nr[i] = make_float4(a, b, c, 0.0f);
        fl = (fl & ~FLAG_HAS_NORMAL) | (h ? FLAG_HAS_NORMAL : 0u);
    }
    fl &= ~FLAG_XO_IS_X;
    other[2 * i] = make_float4(xov.x, xov.y, xov.z, 0.0f);
    st[2 * i] = make_float4(xv.x, xv.y, xv.z, v.x);
    st[2 * i + 1] = make_float4(v.y, v.z, __uint_as_float(fl), 0.0f);
    if (drec ? !tame_d(xv, v, dmax) : !tame(xv, v)) atomicOr(wild, 1u);
}

__global__ void k_check_tame(const float4* __restrict__ st, int64_t n, uint32_t* wild) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s0 = st[2 * i], s1 = st[2 * i + 1];
    if (!tame(mk3(s0.x, s0.y, s0.z), mk3(s0.w, s1.x, s1.y))) atomicOr(wild, 1u);
}

__global__ void k_clear_margin(float4* st, int64_t v0, int64_t v1) {
    const int64_t i = v0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < v1) reinterpret_cast<float*>(st + 2 * i + 1)[3] = 0.0f;
}

__global__ void k_count_contacts(const float4* __restrict__ st, int64_t n, unsigned long long* count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool c = i < n && (__float_as_uint(st[2 * i + 1].z) & FLAG_HAS_NORMAL);
    const unsigned m = __ballot_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

// update_vertex (simulation.cu:253-257): x = x_old = p, so v = (p - p) / dt; the
// stored contact normal is kept
__global__ void k_set_vertices(float4* st, const uint32_t* __restrict__ idx, const float* __restrict__ xyz3, int n,
                               float dt, uint32_t* wild) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t v = idx[k];
    const f3 p = mk3(xyz3[3 * k], xyz3[3 * k + 1], xyz3[3 * k + 2]);
    const f3 vel = divs(sub(p, p), dt);
    const uint32_t fl = (__float_as_uint(st[2 * v + 1].z) & FLAG_HAS_NORMAL) | FLAG_XO_IS_X;
    st[2 * v] = make_float4(p.x, p.y, p.z, vel.x);
    st[2 * v + 1] = make_float4(vel.y, vel.z, __uint_as_float(fl), 0.0f);
    if (!tame(p, vel)) atomicOr(wild, 1u);
}

inline unsigned grid_for(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

namespace {
// Self-test of the staging ring's bounded wait: thread 0 waits on the phase of an
// mbarrier that nothing arrives on; the wait gives up after kWaitNs and the kernel
// records ERR_TIMEOUT and returns (no copy is in flight).
__global__ void k_selftest_mbar_wait(int* err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(smem_addr(&bar), 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait(smem_addr(&bar), 0u)) atomicOr(err, ERR_TIMEOUT);
}
}  // namespace

namespace {
// Every float s of [2^-100, 2^100) (the range where the step takes the packed square
// root and reciprocal) through sqrt_rcp_pair, against __fsqrt_rn(s) and
// __frcp_rn(__fsqrt_rn(s)).  The other lane of each pair carries a different float of
// the range (s with its low mantissa bits reversed), checked too.  cnt[0] = floats
// checked, cnt[1] = mismatches of the root, cnt[2] = of the reciprocal.
__global__ void k_selftest_exact_math(unsigned long long* cnt) {
    unsigned long long n = 0, bad_q = 0, bad_r = 0;
    const uint64_t lo = kExactLo, hi = (uint64_t)kExactLo + kExactSpan;
    for (uint64_t u = lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < hi;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)u;
        const uint32_t b2 = (b & 0xffff0000u) | (__brev(b) >> 16);  // same exponent, other mantissa
        const float sa = __uint_as_float(b), sb = __uint_as_float(b2);
        fp2 q, r;
        sqrt_rcp_pair(pk2(sa, sb), q, r);
        const float qa = __fsqrt_rn(sa), qb = __fsqrt_rn(sb);
        bad_q += (__float_as_uint(lo2(q)) != __float_as_uint(qa)) + (__float_as_uint(hi2(q)) != __float_as_uint(qb));
        bad_r += (__float_as_uint(lo2(r)) != __float_as_uint(__frcp_rn(qa))) +
                 (__float_as_uint(hi2(r)) != __float_as_uint(__frcp_rn(qb)));
        n += 2;
    }
    atomicAdd(&cnt[0], n);
    if (bad_q) atomicAdd(&cnt[1], bad_q);
    if (bad_r) atomicAdd(&cnt[2], bad_r);
}
}  // namespace

cudaError_t launch_selftest_exact_math(unsigned long long* cnt, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_selftest_exact_math<<<sms * 8, 256, 0, s>>>(cnt);
    return cudaGetLastError();
}

cudaError_t launch_selftest_mbar_wait(int* err, cudaStream_t s) {
    k_selftest_mbar_wait<<<1, 32, 0, s>>>(err);
    return cudaGetLastError();
}

void set_step_timing(cudaEvent_t before, cudaEvent_t after) {
    t_before_step = before;
    t_after_step = after;
}

cudaError_t launch_step(const StepArgs& a, int variant, int block, int grid, cudaStream_t s) {
    if (a.n_tiles == 0) return cudaSuccess;
    if (grid <= 0 || grid > a.n_tiles) grid = a.n_tiles;
    switch (block) {
        case 128: return launch_block<128>(a, variant, grid, s);
        case 256: return launch_block<256>(a, variant, grid, s);
        case 512: return launch_block<512>(a, variant, grid, s);
        case 1024: return launch_block<1024>(a, variant, grid, s);
        default: return cudaErrorInvalidValue;
    }
}

int step_smem_bytes(int variant, int win_cap) {
    return (variant & SV_STAGED) ? kBarBytes + 2 * 8 * win_cap : 0;
}

int step_max_ctas_per_sm(int variant, int block, int win_cap) {
    switch (block) {
        case 128: return occupancy_block<128>(variant, win_cap);
        case 256: return occupancy_block<256>(variant, win_cap);
        case 512: return occupancy_block<512>(variant, win_cap);
        case 1024: return occupancy_block<1024>(variant, win_cap);
        default: return 0;
    }
}

cudaError_t launch_query(BvhView v, const float* pts, int n, int* leaf, int* inside, float* dist, float* normal,
                         int* err, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_query<<<grid_for(n, 256), 256, 0, s>>>(v, pts, n, leaf, inside, dist, normal, err);
    return cudaGetLastError();
}

cudaError_t launch_unpack_positions(const float4* state, int64_t n, float* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_unpack_positions<<<grid_for(n, 256), 256, 0, s>>>(state, n, out);
    return cudaGetLastError();
}

cudaError_t launch_unpack_state(const float4* state, const float4* other, const float4* normal, int64_t n, float* x,
                                float* xo, float* nrm, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_unpack_state<<<grid_for(n, 256), 256, 0, s>>>(state, other, normal, n, x, xo, nrm);
    return cudaGetLastError();
}

cudaError_t launch_check_tame(const float4* state, int64_t n, uint32_t* wild, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_check_tame<<<grid_for(n, 256), 256, 0, s>>>(state, n, wild);
    return cudaGetLastError();
}

cudaError_t launch_clear_margin(float4* state, int64_t v0, int64_t v1, cudaStream_t s) {
    if (v1 <= v0) return cudaSuccess;
    k_clear_margin<<<grid_for(v1 - v0, 256), 256, 0, s>>>(state, v0, v1);
    return cudaGetLastError();
}

cudaError_t launch_count_contacts(const float4* state, int64_t n, unsigned long long* count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_count_contacts<<<grid_for(n, 256), 256, 0, s>>>(state, n, count);
    return cudaGetLastError();
}

cudaError_t launch_set_vertices(float4* state, const uint32_t* idx, const float* xyz, int n, float dt, uint32_t* wild,
                                cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_set_vertices<<<grid_for(n, 256), 256, 0, s>>>(state, idx, xyz, n, dt, wild);
    return cudaGetLastError();
}

cudaError_t launch_pack_state(float4* state, float4* other, float4* normal, int64_t n, const float* x, const float* xo,
                              const float* nrm, float dt, int drec, float dmax, uint32_t* wild, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_pack_state<<<grid_for(n, 256), 256, 0, s>>>(state, other, normal, n, x, xo, nrm, dt, drec, dmax, wild);
    return cudaGetLastError();
}

}  // namespace visg
