// visg_lbvh.cu — per-step body LBVH build on the device, in one launch.
//
// Reference (BVHAccel, src/bvh/bvh.cu:154-297; cudaBRT.cu:9-206) builds once per
// body with a device->host->device round trip: expanded boxes and Morton codes on
// the GPU, std::sort + duplicate removal on the CPU, then Karras internal nodes and
// an atomic-counter refit on the GPU.  Here the whole build is one cooperative
// launch of k_rebuild, so it can run every step: persistent CTAs, all resident at
// once, walk its phases, and a grid barrier (every CTA arrives on a counter, then
// waits for the others, bounded) separates phases that read what others wrote:
//   verts   vertex_extend (Mesh.cpp:101-117) v += thickness * n, stored as float4
//           (the same launch voids the query-cache margins of the body's cloth)
//   boxes   expanded triangle boxes (primitive.cu:79-91) and leaf records, three
//           corners gathered as aligned float4; per CTA the union of its boxes
//           with the identity box
//   codes   the Morton frame (identity box U every box: each CTA reduces the CTA
//           unions itself); the Morton code of each box centroid in the frame
//           (bvh.cu:20-41,71-79; bbox.h:97-127); codes that differ from the last
//           build's are listed
//   sort    the stable order by (code, triangle).  When the last build's sorted
//           list is at hand and at most CHG_CAP codes changed (a body that moves
//           rigidly flips a few codes at cell edges), it is merged: the unchanged
//           entries keep their order, every CTA sorts the changed ones in shared
//           memory, and each entry's new position follows from binary searches
//           (phase_merge).  Otherwise four stable LSD radix passes over 8-bit
//           digits, tiles claimed in order, decoupled look-back.
//   unique  keep the first triangle of every distinct code (remove_redundant,
//           Utilities.h:35-55): per-CTA counts, a barrier, then each CTA's offset
//   build   bottom-up radix-tree build fused with the refit, per chunk of 512
//           sorted leaves: each leaf thread climbs with handshakes in shared
//           memory while both children lie in the chunk; the parent of range
//           [l, r] is the boundary with the longer common prefix (delta(l-1,l)
//           vs delta(r,r+1), delta = clz(a ^ b) as cudaBRT.cu:9-19), the second
//           child to arrive merges both boxes into the identity box
//           (calculateBoudingBox, cudaBRT.cu:166-206) and continues.  Each chunk
//           then publishes a summary for the nodes that span chunks; the CTA that
//           finishes the last chunk of a group of 32 sums the group up a level
//   top     one warp per node that spans chunks: its range ends are the nearest
//           boundaries with a smaller delta, its box the union of its leaves'
//           boxes, both read off the chunk summaries
// Nodes are numbered by their split position; the tree is the same binary radix
// tree processInternalNode (cudaBRT.cu:120-161) builds, and visg_export_lbvh
// renumbers it into the reference's layout.  Data one CTA reads after another wrote
// it in the same launch is loaded through L2 (ld.global.cg), never the read-only
// path.  Every wait is bounded; a wait that gives up sets ERR_TIMEOUT, the CTA skips
// the rest of its work (still arriving at each barrier), and the host reports
// VISG_ERR_TIMEOUT.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "visg_internal.cuh"

namespace visg {

namespace {

constexpr int RB = 512;        // threads per CTA: one chunk of leaves, one leaf per thread
constexpr int RW = RB / 32;    // warps per CTA
constexpr int SORT_ITEMS = 4;
constexpr int SORT_TILE = RB * SORT_ITEMS;  // 2048 keys per radix tile
constexpr int RADIX = 256;
constexpr int PASSES = 4;
constexpr int UNIQ_ITEMS = 4;
constexpr int CHG_CAP = 2048;  // changed codes the incremental sort merges
constexpr uint32_t ST_AGG = 1u << 30;
constexpr uint32_t ST_PREFIX = 2u << 30;
constexpr uint32_t ST_VALUE = (1u << 30) - 1u;
constexpr int SPIN_LIMIT = 1 << 22;
constexpr uint64_t kGridWaitNs = 1000000000ull;  // a grid barrier gives up after 1 s
constexpr int BUILD_LEAVES = RB;                 // leaves per chunk
constexpr int NLEV = 4;
constexpr int BIG_DELTA = 64;  // above every delta: a boundary that does not exist

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) { *reinterpret_cast<volatile uint32_t*>(p) = v; }
__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Decoupled look-back: the exclusive prefix of tile `tile` from the status words of
// the tiles before it (tile t's at st0[t * stride]: 0 = not yet published, ST_AGG |
// its own count, ST_PREFIX | its inclusive prefix).  A word only ever goes from 0 to
// AGG to PREFIX, so one read of it stays valid: LB_WINDOW predecessors are read per
// round trip, summed in order down to the first PREFIX; a word still 0 is waited on
// (bounded) and the walk resumes there.
constexpr int LB_WINDOW = 8;
__device__ __forceinline__ uint32_t look_back(const uint32_t* st0, size_t stride, int tile, int* err) {
    uint32_t excl = 0;
    int t = tile - 1, spins = 0;
    while (t >= 0) {
        uint32_t w[LB_WINDOW];
#pragma unroll
        for (int q = 0; q < LB_WINDOW; ++q) w[q] = t - q >= 0 ? ld_volatile(st0 + (size_t)(t - q) * stride) : 0u;
        int q = 0;
        bool done = false;
        for (; q < LB_WINDOW && t - q >= 0; ++q) {
            const uint32_t f = w[q] & ~ST_VALUE;
            if (f == 0u) break;  // not published yet
            excl += w[q] & ST_VALUE;
            if (f == ST_PREFIX) {
                done = true;
                break;
            }
        }
        if (done) break;
        t -= q;
        if (q < LB_WINDOW) {  // stopped at an unpublished tile (tile 0 always publishes a PREFIX)
            if (++spins > SPIN_LIMIT) {
                atomicOr(err, ERR_TIMEOUT);
                break;
            }
            __nanosleep(32);
        }
    }
    return excl;
}

// inclusive scan of one value per thread over the CTA (s_warp: 32 words); the CTA
// total is left in s_warp[RW - 1]
__device__ __forceinline__ uint32_t block_scan_incl(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < RW ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < RW) s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t r = v + (warp > 0 ? s_warp[warp - 1] : 0u);
    __syncthreads();
    return r;
}
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_warp) {
    (void)block_scan_incl(v, s_warp);
    const uint32_t t = s_warp[RW - 1];
    __syncthreads();  // every thread has read it before the next scan writes s_warp
    return t;
}

// ---- arguments and shared memory ------------------------------------------------------------
struct ChunkView {
    int* cmin;
    float4* cbox;
    int2* srec;
    float4* sbox;
    int2* prec;
    float4* pbox;
    int* rcnt;
    int2* top;
    int lev_off[NLEV];
};

struct RebuildArgs {
    const float* xyz;
    const float* nrm;  // null: no thickness push
    const uint32_t* tris;
    int nv, nt;
    float thickness, depth;
    int coherent;  // the last build's sorted list and codes may be reused
    int tiles_sort;
    float4* verts;
    float4* tri_box;
    float4* tri_leaf;
    uint32_t* codes;
    uint32_t* keys[2];
    uint32_t* vals[2];
    uint32_t* ucode;
    uint32_t* utri;
    Node* nodes;
    float4* leaves;
    int2* range;
    BvhRoot* root;
    ChunkView cv;
    uint32_t* ghist;   // PASSES x RADIX digit counts
    uint32_t* sstat;   // PASSES x tiles_sort x RADIX look-back status words
    uint32_t* scount;  // PASSES tile counters
    float* part;       // 8 per CTA: its box union (min xyz, max xyz)
    uint32_t* ucnt;    // per CTA: distinct codes in its slice of the sorted list
    uint32_t* chg;     // [0] changed codes, then {triangle, new code, old code} x CHG_CAP
    uint32_t* sync;    // [0] barrier arrivals, [1] CTAs finished (both 0 between launches)
    uint32_t* gdone;   // per summary entry of levels 1..3: its member entries finished
    int n_entries;     // summary entries of all levels
    int* err;
    float4* margin_state;  // cloth records whose query-cache margins the moved body voids
    int64_t m0, m1;        // (vertices [m0, m1): their margin words are cleared)
};

struct BuildSmem {
    uint32_t flag[BUILD_LEAVES];  // bit 0: child A arrived, bit 1: child B
    // per node and side (A, B): lo (w = link), hi (w = far range end)
    float4 lo[BUILD_LEAVES][2], hi[BUILD_LEAVES][2];
    int delta[BUILD_LEAVES + 4];  // delta of boundary j at j - c0 + 1
    int wmin[RW], wsr[RW], wpr[RW], wtop[RW];  // per warp
    float4 wlo[RW], whi[RW];
    // per warp, over the warps before (x*p) / after (x*s) it
    int xpm[RW], xsm[RW], xos[RW], xop[RW], xot[RW];
    float4 xplo[RW], xphi[RW], xslo[RW], xshi[RW];
    int nrec[4];
};
struct SortSmem {
    uint32_t whist[RW][RADIX + 1];
    uint32_t tstart[RADIX];
    uint32_t gbase[RADIX];
    uint32_t keys[SORT_TILE];
    uint32_t vals[SORT_TILE];
};
struct MergeSmem {
    unsigned long long knew[CHG_CAP];  // changed entries by (new code, triangle)
    unsigned long long kold[CHG_CAP];  // the same entries by (old code, triangle)
};
constexpr size_t smax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kSmemBytes = smax(sizeof(BuildSmem), smax(sizeof(SortSmem), sizeof(MergeSmem)));

// ---- grid barrier ---------------------------------------------------------------------------
// Every CTA arrives on sync[0] and waits until it holds `target` (gridDim.x per
// barrier so far).  A CTA whose earlier wait gave up (ok false) still arrives, so
// the others are not held, but does not wait.  Returns whether this CTA may go on.
__device__ bool grid_barrier(uint32_t* ctr, uint32_t& target, bool ok, int* err, int* s_ok) {
    __syncthreads();
    target += gridDim.x;
    if (threadIdx.x == 0) {
        __threadfence();  // this CTA's writes before its arrival
        atomicAdd(ctr, 1u);
        int good = ok ? 1 : 0;
        if (good && ld_volatile(ctr) < target) {
            const uint64_t t0 = now_ns();
            while (ld_volatile(ctr) < target) {
                if (now_ns() - t0 > kGridWaitNs) {
                    atomicOr(err, ERR_TIMEOUT);
                    good = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();  // the others' writes before this CTA's reads
        *s_ok = good;
    }
    __syncthreads();
    return *s_ok != 0;
}

// ---- boxes ------------------------------------------------------------------------------------
__device__ __forceinline__ f3 pushed(const RebuildArgs& A, uint32_t v) {  // vertex_extend
    float x = __ldg(A.xyz + 3 * v), y = __ldg(A.xyz + 3 * v + 1), z = __ldg(A.xyz + 3 * v + 2);
    if (A.nrm) {
        x = __fadd_rn(x, __fmul_rn(A.thickness, __ldg(A.nrm + 3 * v)));
        y = __fadd_rn(y, __fmul_rn(A.thickness, __ldg(A.nrm + 3 * v + 1)));
        z = __fadd_rn(z, __fmul_rn(A.thickness, __ldg(A.nrm + 3 * v + 2)));
    }
    return mk3(x, y, z);
}

__device__ __forceinline__ void box_add(f3& lo, f3& hi, f3 p) {
    lo.x = fminf(lo.x, p.x); lo.y = fminf(lo.y, p.y); lo.z = fminf(lo.z, p.z);
    hi.x = fmaxf(hi.x, p.x); hi.y = fmaxf(hi.y, p.y); hi.z = fmaxf(hi.z, p.z);
}

// min (k < 3) / max (k >= 3) of r[6] over the CTA, into s_red[6] (all threads)
__device__ __forceinline__ void block_box_reduce(float r[6], float* s_red /* 6 * RW */) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = fminf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
#pragma unroll
        for (int k = 3; k < 6; ++k) r[k] = fmaxf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 6; ++k) s_red[k * RW + warp] = r[k];
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        float v = s_red[k * RW];
        for (int w = 1; w < RW; ++w) v = k < 3 ? fminf(v, s_red[k * RW + w]) : fmaxf(v, s_red[k * RW + w]);
        s_red[k * RW] = v;
    }
    __syncthreads();
}

// the pushed vertices, as float4 (one aligned load per corner in phase_boxes); the
// query-cache margins of the body's cloth vertices are voided (the body moves)
__device__ void phase_verts(const RebuildArgs& A) {
    for (int v = blockIdx.x * RB + threadIdx.x; v < A.nv; v += gridDim.x * RB) {
        const f3 p = pushed(A, (uint32_t)v);
        A.verts[v] = make_float4(p.x, p.y, p.z, 0.0f);
    }
    if (A.margin_state)
        for (int64_t i = A.m0 + (int64_t)blockIdx.x * RB + threadIdx.x; i < A.m1; i += (int64_t)gridDim.x * RB)
            reinterpret_cast<float*>(A.margin_state + 2 * i + 1)[3] = 0.0f;
}

constexpr int BOX_BATCH = 3;  // triangles a thread loads before it computes any

// each triangle's expanded box (BBox(v0).expand(v1).expand(v2) and the three
// corners pushed inward by depth * n) and leaf record; the CTA's union of its boxes
// with the identity box in part[8 * cta]
__device__ void phase_boxes(const RebuildArgs& A, float* s_red) {
    const int stride = gridDim.x * RB;
    f3 lo = mk3(100.0f, 100.0f, 100.0f), hi = mk3(-100.0f, -100.0f, -100.0f);
    for (int base = blockIdx.x * RB + threadIdx.x; base < A.nt; base += BOX_BATCH * stride) {
        uint32_t idx[BOX_BATCH][3];
#pragma unroll
        for (int q = 0; q < BOX_BATCH; ++q) {
            const int t = base + q * stride;
#pragma unroll
            for (int c = 0; c < 3; ++c) idx[q][c] = t < A.nt ? __ldg(A.tris + 3 * t + c) : 0u;
        }
        float4 w[BOX_BATCH][3];
#pragma unroll
        for (int q = 0; q < BOX_BATCH; ++q)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                // vertex indices come from the caller: one out of range is recorded and
                // read as vertex 0, so no load leaves the vertex array (the build's
                // result is then reported as failed)
                uint32_t v = idx[q][c];
                if (v >= (uint32_t)A.nv) {
                    if (base + q * stride < A.nt) atomicOr(A.err, ERR_INDEX);
                    v = 0u;
                }
                w[q][c] = __ldcg(A.verts + v);
            }
#pragma unroll
        for (int q = 0; q < BOX_BATCH; ++q) {
            const int t = base + q * stride;
            if (t >= A.nt) break;
            const f3 v0 = xyz(w[q][0]), v1 = xyz(w[q][1]), v2 = xyz(w[q][2]);
            const f3 n = normalize(cross(sub(v1, v0), sub(v2, v0)));  // Primitive::d_get_normal
            f3 blo = v0, bhi = v0;
            box_add(blo, bhi, v1);
            box_add(blo, bhi, v2);
            const f3 dn = mul(A.depth, n);
            box_add(blo, bhi, sub(v0, dn));
            box_add(blo, bhi, sub(v1, dn));
            box_add(blo, bhi, sub(v2, dn));
            A.tri_box[2 * t] = make_float4(blo.x, blo.y, blo.z, 0.0f);
            A.tri_box[2 * t + 1] = make_float4(bhi.x, bhi.y, bhi.z, 0.0f);
            A.tri_leaf[2 * t] = make_float4(v0.x, v0.y, v0.z, n.x);
            A.tri_leaf[2 * t + 1] = make_float4(n.y, n.z, __int_as_float(t), 0.0f);
            box_add(lo, hi, blo);
            box_add(lo, hi, bhi);
        }
    }
    float r[6] = {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
    block_box_reduce(r, s_red);
    if (threadIdx.x < 6) A.part[8 * blockIdx.x + threadIdx.x] = s_red[threadIdx.x * RW];
}

// ---- codes ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {  // bvh.cu:20-27
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// the frame from the CTA unions; each triangle's code; with `listing`, the triangles
// whose code changed go to the change list (at most CHG_CAP are stored)
__device__ void phase_codes(const RebuildArgs& A, bool listing, float* s_red, float* s_frame) {
    float r[6] = {100.0f, 100.0f, 100.0f, -100.0f, -100.0f, -100.0f};
    for (int c = threadIdx.x; c < (int)gridDim.x; c += RB) {
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = fminf(r[k], __ldcg(A.part + 8 * c + k));
#pragma unroll
        for (int k = 3; k < 6; ++k) r[k] = fmaxf(r[k], __ldcg(A.part + 8 * c + k));
    }
    block_box_reduce(r, s_red);
    if (threadIdx.x < 6) s_frame[threadIdx.x] = s_red[threadIdx.x * RW];
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        A.root->frame_lo = make_float4(s_frame[0], s_frame[1], s_frame[2], 0.0f);
        A.root->frame_hi = make_float4(s_frame[3], s_frame[4], s_frame[5], 0.0f);
    }
    const f3 fmn = mk3(s_frame[0], s_frame[1], s_frame[2]);
    const f3 ext = sub(mk3(s_frame[3], s_frame[4], s_frame[5]), fmn);
    const bool flat = length(ext) == 0.0f;
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * RB;
    for (int base = blockIdx.x * RB; base < A.nt; base += 2 * stride) {  // warp-uniform bounds
        // both triangles' loads first
        float4 blo[2], bhi[2];
        uint32_t old[2] = {0u, 0u};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int t = base + q * stride + threadIdx.x;
            if (t < A.nt) {
                blo[q] = __ldcg(A.tri_box + 2 * t);
                bhi[q] = __ldcg(A.tri_box + 2 * t + 1);
                if (listing) old[q] = A.codes[t];
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int t = base + q * stride + threadIdx.x;
            bool changed = false;
            uint32_t code = 0u;
            if (t < A.nt) {
                const f3 c = divs(add(xyz(blo[q]), xyz(bhi[q])), 2.0f);  // BBox::centroid
                f3 u = mk3(0.0f, 0.0f, 0.0f);
                if (!flat) u = divv(sub(c, fmn), ext);  // BBox::getUnitcubePosOf
                const float x = fminf(fmaxf(__fmul_rn(u.x, 1024.0f), 0.0f), 1023.0f);
                const float y = fminf(fmaxf(__fmul_rn(u.y, 1024.0f), 0.0f), 1023.0f);
                const float z = fminf(fmaxf(__fmul_rn(u.z, 1024.0f), 0.0f), 1023.0f);
                code = expand_bits((uint32_t)x) * 4u + expand_bits((uint32_t)y) * 2u + expand_bits((uint32_t)z);
                A.codes[t] = code;
                changed = listing && old[q] != code;
            }
            const unsigned m = __ballot_sync(0xffffffffu, changed);
            if (m) {
                const int leader = __ffs(m) - 1;
                uint32_t b0 = 0;
                if (lane == leader) b0 = atomicAdd(A.chg, (uint32_t)__popc(m));
                b0 = __shfl_sync(0xffffffffu, b0, leader);
                const uint32_t k = b0 + (uint32_t)__popc(m & ((1u << lane) - 1u));
                if (changed && k < (uint32_t)CHG_CAP) {
                    A.chg[1 + 3 * k] = (uint32_t)t;
                    A.chg[2 + 3 * k] = code;
                    A.chg[3 + 3 * k] = old[q];
                }
            }
        }
    }
}

// ---- sort: incremental merge --------------------------------------------------------------------
__device__ __forceinline__ unsigned long long key64(uint32_t code, uint32_t tri) {
    return ((unsigned long long)code << 32) | tri;
}
// entries of a[0, n) below x (a ascending)
__device__ __forceinline__ int lower_bound64(const unsigned long long* a, int n, unsigned long long x) {
    int lo = 0, len = n;
    while (len > 0) {
        const int h = len >> 1;
        if (a[lo + h] < x) {
            lo += h + 1;
            len -= h + 1;
        } else {
            len = h;
        }
    }
    return lo;
}

// Merge of the nc changed entries into the last build's sorted list ko/vo (all nt
// triangles by (code, triangle), old codes): every CTA sorts the changed entries by
// new key (knew) and by old key (kold), then walks its slice of the old list.  For
// old slot s with key k_s, q(s) = #kold < k_s and r(s) = #knew < k_s.  An unchanged
// entry keeps its code, so its key is k_s and its new position is s - q(s) (the
// unchanged entries before it) + r(s) (the changed entries that now sort before
// it).  Changed entry j with r(s) <= j < r(s + 1) lies strictly between k_s and
// k_(s+1): s + 1 - q(s + 1) unchanged entries sort before it, j changed ones, so its
// position is j + s + 1 - q(s + 1).  Changed entries below the first old key go to
// positions j (CTA 0).  Positions are a permutation of [0, nt); each is checked.
__device__ void phase_merge(const RebuildArgs& A, int nc, const uint32_t* ko, const uint32_t* vo, uint32_t* kn,
                            uint32_t* vn, MergeSmem& S) {
    int P = 1;
    while (P < nc) P <<= 1;
    for (int k = threadIdx.x; k < P; k += RB) {
        if (k < nc) {
            const uint32_t t = __ldcg(A.chg + 1 + 3 * k);
            S.knew[k] = key64(__ldcg(A.chg + 2 + 3 * k), t);
            S.kold[k] = key64(__ldcg(A.chg + 3 + 3 * k), t);
        } else {
            S.knew[k] = S.kold[k] = ~0ull;
        }
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)  // bitonic sort of both arrays, ascending
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += RB) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const unsigned long long a = S.knew[i], b = S.knew[l];
                    if ((a > b) == up) {
                        S.knew[i] = b;
                        S.knew[l] = a;
                    }
                    const unsigned long long c = S.kold[i], d = S.kold[l];
                    if ((c > d) == up) {
                        S.kold[i] = d;
                        S.kold[l] = c;
                    }
                }
            }
            __syncthreads();
        }
    const int nt = A.nt;
    const int per = (nt + gridDim.x - 1) / gridDim.x;
    const int a = blockIdx.x * per, b = min(nt, a + per);
    constexpr int MB = 3;  // slots a thread loads before it searches
    for (int s0 = a + threadIdx.x; s0 < b; s0 += MB * RB) {
        unsigned long long ks[MB], k1[MB];
#pragma unroll
        for (int u = 0; u < MB; ++u) {
            const int s = s0 + u * RB;
            ks[u] = s < b ? key64(ko[s], vo[s]) : ~0ull;
            k1[u] = s < b && s + 1 < nt ? key64(ko[s + 1], vo[s + 1]) : ~0ull;
        }
#pragma unroll
        for (int u = 0; u < MB; ++u) {
            const int s = s0 + u * RB;
            if (s >= b) break;
            const int q = lower_bound64(S.kold, nc, ks[u]);
            const int r = lower_bound64(S.knew, nc, ks[u]);
            if (!(q < nc && S.kold[q] == ks[u])) {  // unchanged
                const int pos = s - q + r;
                if ((unsigned)pos < (unsigned)nt) {
                    kn[pos] = (uint32_t)(ks[u] >> 32);
                    vn[pos] = (uint32_t)ks[u];
                }
            }
            int r1 = nc, q1 = nc;
            if (s + 1 < nt) {
                r1 = lower_bound64(S.knew, nc, k1[u]);
                q1 = lower_bound64(S.kold, nc, k1[u]);
            }
            for (int j = r; j < r1; ++j) {
                const int pos = j + s + 1 - q1;
                if ((unsigned)pos < (unsigned)nt) {
                    kn[pos] = (uint32_t)(S.knew[j] >> 32);
                    vn[pos] = (uint32_t)S.knew[j];
                }
            }
        }
    }
    if (blockIdx.x == 0 && nt > 0) {
        const int r0 = lower_bound64(S.knew, nc, key64(ko[0], vo[0]));
        for (int j = threadIdx.x; j < r0; j += RB) {
            kn[j] = (uint32_t)(S.knew[j] >> 32);
            vn[j] = (uint32_t)S.knew[j];
        }
    }
}

// ---- sort: radix passes ------------------------------------------------------------------------
// digit counts of all four passes (grid-stride over the codes, per CTA in shared memory)
__device__ void phase_hist(const RebuildArgs& A, uint32_t* s_hist /* PASSES * RADIX */) {
    for (int k = threadIdx.x; k < PASSES * RADIX; k += RB) s_hist[k] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * RB; base < A.nt; base += gridDim.x * RB) {
        const int t = base + threadIdx.x;
        const bool ok = t < A.nt;
        const uint32_t code = ok ? __ldcg(A.codes + t) : 0u;
        // the two high digits are nearly constant across neighbouring triangles, so
        // their lanes add once per equal digit
#pragma unroll
        for (int p = 0; p < PASSES; ++p) {
            const uint32_t dig = (code >> (8 * p)) & 255u;
            if (p < 2) {
                if (ok) atomicAdd(&s_hist[p * RADIX + dig], 1u);
            } else {
                const uint32_t peers = __match_any_sync(0xffffffffu, ok ? dig : RADIX);
                if (ok && lane == __ffs(peers) - 1) atomicAdd(&s_hist[p * RADIX + dig], (uint32_t)__popc(peers));
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < PASSES * RADIX; k += RB) {
        const uint32_t v = s_hist[k];
        if (v) atomicAdd(&A.ghist[k], v);
    }
}

// One tile of a stable LSD pass over 8-bit digit (key >> shift) & 255.  Tiles are
// claimed in order through a counter, so every tile a CTA waits on belongs to a CTA
// that is already at work on it: the look-back always terminates.
__device__ void sort_tile(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, int n, int shift,
                          const uint32_t* ghist, uint32_t* status, int tile, SortSmem& S, uint32_t* s_scan, int* err) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < RW * (RADIX + 1); k += RB) (&S.whist[0][0])[k] = 0;
    __syncthreads();
    const int base = tile * SORT_TILE + warp * (32 * SORT_ITEMS);
    uint32_t key[SORT_ITEMS], val[SORT_ITEMS], rank[SORT_ITEMS];
    int dig[SORT_ITEMS];
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        const int idx = base + j * 32 + lane;  // warp-striped: j-major order is input order
        if (idx < n) {
            key[j] = __ldcg(kin + idx);
            val[j] = vin ? __ldcg(vin + idx) : (uint32_t)idx;
            dig[j] = (int)((key[j] >> shift) & 255u);
        } else {
            key[j] = 0u;
            val[j] = 0u;
            dig[j] = RADIX;  // padding: own bucket, never written
        }
    }
    // stable rank of every key among equal digits of this warp, in input order
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        const uint32_t peers = __match_any_sync(0xffffffffu, dig[j]);
        const int leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (lane == leader) {
            before = S.whist[warp][dig[j]];
            S.whist[warp][dig[j]] = before + __popc(peers);
        }
        before = __shfl_sync(0xffffffffu, before, leader);
        rank[j] = before + __popc(peers & ((1u << lane) - 1u));
        __syncwarp();
    }
    __syncthreads();
    // thread d < RADIX owns digit d: warp-exclusive prefixes and the tile count
    const int d = tid;
    uint32_t tcount = 0;
    if (d < RADIX) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < RW; ++w) {
            const uint32_t c = S.whist[w][d];
            S.whist[w][d] = run;
            run += c;
        }
        tcount = run;
    }
    const uint32_t tincl = block_scan_incl(tcount, s_scan);
    if (d < RADIX) S.tstart[d] = tincl - tcount;
    const uint32_t gh = d < RADIX ? __ldcg(ghist + d) : 0u;
    const uint32_t goff = block_scan_incl(gh, s_scan) - gh;
    // publish the tile's count of digit d, then look back for the exclusive prefix
    if (d < RADIX) {
        uint32_t excl = 0;
        uint32_t* st = status + (size_t)tile * RADIX + d;
        if (tile == 0) {
            st_volatile(st, ST_PREFIX | tcount);
        } else {
            st_volatile(st, ST_AGG | tcount);
            excl = look_back(status + d, RADIX, tile, err);
            st_volatile(st, ST_PREFIX | ((excl + tcount) & ST_VALUE));
        }
        S.gbase[d] = goff + excl;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        if (dig[j] < RADIX) {
            const uint32_t pos = S.tstart[dig[j]] + S.whist[warp][dig[j]] + rank[j];
            S.keys[pos] = key[j];
            S.vals[pos] = val[j];
        }
    }
    __syncthreads();
    const int tile_n = min(SORT_TILE, n - tile * SORT_TILE);
    for (int p = tid; p < tile_n; p += RB) {
        const uint32_t k = S.keys[p];
        const uint32_t dd = (k >> shift) & 255u;
        const uint32_t o = S.gbase[dd] + (uint32_t)p - S.tstart[dd];
        if (o < (uint32_t)n) {  // always true unless a look-back gave up
            kout[o] = k;
            vout[o] = S.vals[p];
        }
    }
    __syncthreads();
}

__device__ void phase_sort_pass(const RebuildArgs& A, int p, SortSmem& S, uint32_t* s_scan, int* s_claim) {
    const uint32_t* kin = p == 0 ? A.codes : A.keys[(p - 1) & 1];
    const uint32_t* vin = p == 0 ? nullptr : A.vals[(p - 1) & 1];
    for (;;) {
        if (threadIdx.x == 0) *s_claim = (int)atomicAdd(A.scount + p, 1u);
        __syncthreads();
        const int tile = *s_claim;
        __syncthreads();
        if (tile >= A.tiles_sort) break;
        sort_tile(kin, vin, A.keys[p & 1], A.vals[p & 1], A.nt, 8 * p, A.ghist + p * RADIX,
                  A.sstat + (size_t)p * A.tiles_sort * RADIX, tile, S, s_scan, A.err);
    }
}

// ---- unique ------------------------------------------------------------------------------------
// CTA c takes positions [c * per, (c + 1) * per) of the sorted list; position p is a
// leaf when p == 0 or its code differs from p - 1's
__device__ __forceinline__ bool first_of_code(const uint32_t* K, int p) {
    return p == 0 || __ldcg(K + p) != __ldcg(K + p - 1);
}

__device__ void phase_unique_count(const RebuildArgs& A, const uint32_t* K, uint32_t* s_scan) {
    const int per = (A.nt + gridDim.x - 1) / gridDim.x;
    const int a = blockIdx.x * per, b = min(A.nt, a + per);
    uint32_t c = 0;
    for (int p = a + threadIdx.x; p < b; p += RB) c += first_of_code(K, p) ? 1u : 0u;
    const uint32_t tot = block_sum(c, s_scan);
    if (threadIdx.x == 0) A.ucnt[blockIdx.x] = tot;
}

// the leaves of this CTA's slice at its offset (the counts of the CTAs before it);
// returns the number of leaves in all
__device__ int phase_unique_write(const RebuildArgs& A, const uint32_t* K, const uint32_t* V, uint32_t* s_scan) {
    uint32_t before = 0, all = 0;
    for (int c = threadIdx.x; c < (int)gridDim.x; c += RB) {
        const uint32_t v = __ldcg(A.ucnt + c);
        all += v;
        if (c < (int)blockIdx.x) before += v;
    }
    before = block_sum(before, s_scan);
    all = block_sum(all, s_scan);
    const int per = (A.nt + gridDim.x - 1) / gridDim.x;
    const int a = blockIdx.x * per, b = min(A.nt, a + per);
    uint32_t off = before;
    for (int base = a; base < b; base += RB * UNIQ_ITEMS) {
        const int p0 = base + threadIdx.x * UNIQ_ITEMS;
        uint32_t fl = 0;
#pragma unroll
        for (int j = 0; j < UNIQ_ITEMS; ++j)
            if (p0 + j < b && first_of_code(K, p0 + j)) fl |= 1u << j;
        const uint32_t cnt = __popc(fl);
        const uint32_t incl = block_scan_incl(cnt, s_scan);
        const uint32_t tile_total = s_scan[RW - 1];
        uint32_t o = off + incl - cnt;
#pragma unroll
        for (int j = 0; j < UNIQ_ITEMS; ++j)
            if (fl & (1u << j)) {
                if (o < (uint32_t)A.nt) {
                    A.ucode[o] = __ldcg(K + p0 + j);
                    A.utri[o] = __ldcg(V + p0 + j);
                }
                ++o;
            }
        off += tile_total;
        __syncthreads();  // s_scan is read above before the next scan overwrites it
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) A.root->n_leaves = (int)min(all, (uint32_t)A.nt);
    return (int)min(all, (uint32_t)A.nt);
}

// ---- build ---------------------------------------------------------------------------------------
__device__ __forceinline__ int delta_at(const uint32_t* c, int i, int j, int n) {
    return (j < 0 || j >= n) ? -1 : __clz((int)(__ldcg(c + i) ^ __ldcg(c + j)));
}

// identity box (min +100, max -100) expanded by child A then child B
__device__ __forceinline__ void merge_ab(float4 alo, float4 ahi, float4 blo, float4 bhi, float4& lo, float4& hi) {
    lo = make_float4(fminf(fminf(100.0f, alo.x), blo.x), fminf(fminf(100.0f, alo.y), blo.y),
                     fminf(fminf(100.0f, alo.z), blo.z), 0.0f);
    hi = make_float4(fmaxf(fmaxf(-100.0f, ahi.x), bhi.x), fmaxf(fmaxf(-100.0f, ahi.y), bhi.y),
                     fmaxf(fmaxf(-100.0f, ahi.z), bhi.z), 0.0f);
}

// The child (lo, hi, link) over leaves [l, r] enters its parent g: its side of the
// node and of the node's leaf range.  hi.w carries delta at the boundary beyond the
// child's far end (l - 1 for child A, r for child B).
__device__ __forceinline__ void write_side(Node* nodes, int2* range, int g, bool is_a, float4 lo, float4 hi, int link,
                                           int l, int r, int dfar) {
    if (is_a) {
        nodes[g].a_lo = make_float4(lo.x, lo.y, lo.z, __int_as_float(link));
        nodes[g].a_hi = make_float4(hi.x, hi.y, hi.z, __int_as_float(dfar));
        range[g].x = l;  // leaf ranges of the nodes (read by the export)
    } else {
        nodes[g].b_lo = make_float4(lo.x, lo.y, lo.z, __int_as_float(link));
        nodes[g].b_hi = make_float4(hi.x, hi.y, hi.z, __int_as_float(dfar));
        range[g].y = r;
    }
}

// box union (fminf / fmaxf: exact, so any grouping gives the same box)
__device__ __forceinline__ void box_union(float4& lo, float4& hi, float4 lo2, float4 hi2) {
    lo = make_float4(fminf(lo.x, lo2.x), fminf(lo.y, lo2.y), fminf(lo.z, lo2.z), 0.0f);
    hi = make_float4(fmaxf(hi.x, hi2.x), fmaxf(hi.y, hi2.y), fmaxf(hi.z, hi2.z), 0.0f);
}
__device__ __forceinline__ float4 ident_lo() { return make_float4(100.0f, 100.0f, 100.0f, 0.0f); }
__device__ __forceinline__ float4 ident_hi() { return make_float4(-100.0f, -100.0f, -100.0f, 0.0f); }
__device__ __forceinline__ float4 shfl_f4(float4 v, int o, bool up) {
    return up ? make_float4(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o),
                            __shfl_up_sync(0xffffffffu, v.z, o), 0.0f)
              : make_float4(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o),
                            __shfl_down_sync(0xffffffffu, v.z, o), 0.0f);
}
__device__ __forceinline__ void warp_box_reduce(float4& lo, float4& hi) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float4 l2 = make_float4(__shfl_xor_sync(0xffffffffu, lo.x, o), __shfl_xor_sync(0xffffffffu, lo.y, o),
                                      __shfl_xor_sync(0xffffffffu, lo.z, o), 0.0f);
        const float4 h2 = make_float4(__shfl_xor_sync(0xffffffffu, hi.x, o), __shfl_xor_sync(0xffffffffu, hi.y, o),
                                      __shfl_xor_sync(0xffffffffu, hi.z, o), 0.0f);
        box_union(lo, hi, l2, h2);
    }
}

// entries of each level for n leaves
__device__ __forceinline__ void level_counts(int n, int cnt[NLEV]) {
    cnt[0] = (n + BUILD_LEAVES - 1) / BUILD_LEAVES;
#pragma unroll
    for (int v = 1; v < NLEV; ++v) cnt[v] = (cnt[v - 1] + 31) / 32;
}

// Bottom-up build of the chunk-local nodes, and the chunk summaries.  The CTA owns
// the BUILD_LEAVES sorted leaves [c0, c1) of `chunk` and stages delta of the
// boundaries c0 - 1 .. c1 - 1.  The climb goes through the nodes split inside the
// chunk (c0 <= g <= c1 - 2) in shared memory only: each child leaves its box, link
// and far range end in its side of the node's slot; the first to arrive stops, the
// second merges (A then B) and climbs on.  After the barrier the nodes both of
// whose children arrived are written out; a climb that stopped at a node whose
// other child lies in another chunk, or at a node split outside the chunk, writes
// its side into that node.  The remaining nodes span chunks; phase_top finishes them
// from the chunk summaries written here:
//   * the boundaries that can end such a node's range inside this chunk: the strict
//     suffix minima of delta (the nearest smaller delta to the left of a node
//     further right) and the strict prefix minima (to the right of a node further
//     left), at most 30 each, with the union of the chunk's leaf boxes beyond /
//     up to each of them;
//   * the chunk's min delta and leaf box union;
//   * the nodes of the chunk that span chunks (no smaller delta on one side inside
//     the chunk, and the boundary to the next chunk).
__device__ void build_chunk(const RebuildArgs& A, int chunk, int n, BuildSmem& S) {
    const ChunkView& cv = A.cv;
    const int tid = (int)threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nt = A.nt;
    const int c0 = chunk * BUILD_LEAVES;
    const int c1 = min(c0 + BUILD_LEAVES, n);
    S.flag[tid] = 0u;
    const int i = c0 + tid;
    int l = i, r = i, link = ~i;  // the current subtree: leaf range, link
    float4 lo = ident_lo(), hi = ident_hi();
    bool live = i < n;  // still climbing
    int pend = -1;      // node where the climb stopped as the first local arrival
    int out = -1;       // node split outside the chunk where the climb stopped
    int dl = -1, dr = -1;
    bool is_a = false;
    uint32_t t = 0;  // the leaf's triangle
    if (live) {
        t = min(__ldcg(A.utri + i), (uint32_t)(nt - 1));
        lo = __ldcg(A.tri_box + 2 * t);
        hi = __ldcg(A.tri_box + 2 * t + 1);
    }
    {
        const int j = c0 + tid;
        S.delta[tid + 1] = delta_at(A.ucode, j, j + 1, n);  // -1 beyond the last leaf
        if (tid == 0) S.delta[0] = c0 < n ? delta_at(A.ucode, c0, c0 - 1, n) : -1;
    }
    __syncthreads();
    if (live && n == 1) {
        A.root->root = -1;
        A.root->top_lo = lo;
        A.root->top_hi = hi;
        live = false;
    }
    const float4 leaf_lo = lo, leaf_hi = hi;  // identity box for threads past the last leaf
    int level = 0;
    while (live) {
        if (++level > 64) {  // a climb is at most 31 levels over distinct 30-bit codes
            atomicOr(A.err, ERR_TIMEOUT);
            break;
        }
        dl = S.delta[l - c0];      // boundary l - 1
        dr = S.delta[r - c0 + 1];  // boundary r
        is_a = dr > dl;            // the parent extends to the right: this node is child A
        const int g = is_a ? r : l - 1;
        if (g < c0 || g > c1 - 2) {  // split outside the chunk
            out = g;
            break;
        }
        const int k = g - c0, side = is_a ? 0 : 1;
        S.lo[k][side] = make_float4(lo.x, lo.y, lo.z, __int_as_float(link));
        S.hi[k][side] = make_float4(hi.x, hi.y, hi.z, __int_as_float(is_a ? l : r));
        __threadfence_block();
        if (atomicOr(&S.flag[k], 1u << side) == 0u) {  // first to arrive: the sibling may be in another chunk
            pend = g;
            break;
        }
        __threadfence_block();
        // second to arrive: the sibling's side of the slot is complete
        const float4 olo = S.lo[k][side ^ 1], ohi = S.hi[k][side ^ 1];
        const int far = __float_as_int(ohi.w);
        if (is_a) {
            merge_ab(lo, hi, olo, ohi, lo, hi);
            r = far;
        } else {
            merge_ab(olo, ohi, lo, hi, lo, hi);
            l = far;
        }
        link = g;
        if (l == 0 && r == n - 1) {
            A.root->root = g;
            A.root->top_lo = lo;
            A.root->top_hi = hi;
            break;
        }
    }
    __syncthreads();
    if (i < n) {
        A.leaves[2 * i] = __ldcg(A.tri_leaf + 2 * t);
        A.leaves[2 * i + 1] = __ldcg(A.tri_leaf + 2 * t + 1);
    }
    // nodes of the chunk whose children both arrived here
    {
        const int g = c0 + tid;
        if (g <= c1 - 2 && S.flag[tid] == 3u) {
            const float4 alo = S.lo[tid][0], ahi = S.hi[tid][0], blo = S.lo[tid][1], bhi = S.hi[tid][1];
            const int la = __float_as_int(ahi.w), rb = __float_as_int(bhi.w);
            A.nodes[g].a_lo = alo;
            A.nodes[g].a_hi = make_float4(ahi.x, ahi.y, ahi.z, __int_as_float(S.delta[la - c0]));
            A.nodes[g].b_lo = blo;
            A.nodes[g].b_hi = make_float4(bhi.x, bhi.y, bhi.z, __int_as_float(S.delta[rb - c0 + 1]));
            A.range[g] = make_int2(la, rb);
        }
    }
    // a climb that stopped at a node another chunk completes: its side, in the node
    {
        int g = out;
        if (g < 0 && pend >= 0 && S.flag[pend - c0] != 3u) g = pend;
        if (g >= 0) write_side(A.nodes, A.range, g, is_a, lo, hi, link, l, r, is_a ? dl : dr);
    }
    if (c0 < n) {
        // thread tid: boundary j = c0 + tid (delta dk, BIG_DELTA past the last boundary)
        // and leaf c0 + tid (its box, the identity box past the last leaf)
        const int j = c0 + tid;
        const int dk = j <= n - 2 ? S.delta[tid + 1] : BIG_DELTA;
        int pm = dk, sm = dk;  // inclusive prefix / suffix min over the warp
        float4 plo = leaf_lo, phi = leaf_hi, slo = leaf_lo, shi = leaf_hi;  // inclusive prefix / suffix unions
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int a = __shfl_up_sync(0xffffffffu, pm, o), b = __shfl_down_sync(0xffffffffu, sm, o);
            const float4 al = shfl_f4(plo, o, true), ah = shfl_f4(phi, o, true);
            const float4 bl = shfl_f4(slo, o, false), bh = shfl_f4(shi, o, false);
            if (lane >= o) {
                pm = min(pm, a);
                box_union(plo, phi, al, ah);
            }
            if (lane + o < 32) {
                sm = min(sm, b);
                box_union(slo, shi, bl, bh);
            }
        }
        if (lane == 31) {
            S.wmin[warp] = pm;
            S.wlo[warp] = plo;
            S.whi[warp] = phi;
        }
        __syncthreads();
        if (warp == 0) {  // exclusive prefix / suffix over the warps, lane w for warp w
            const bool in = lane < RW;
            int a = in ? S.wmin[lane] : BIG_DELTA, b = a;  // inclusive scans, then shifted
            float4 al = in ? S.wlo[lane] : ident_lo(), ah = in ? S.whi[lane] : ident_hi();
            float4 bl = al, bh = ah;
#pragma unroll
            for (int o = 1; o < RW; o <<= 1) {
                const int pa = __shfl_up_sync(0xffffffffu, a, o), pb = __shfl_down_sync(0xffffffffu, b, o);
                const float4 pal = shfl_f4(al, o, true), pah = shfl_f4(ah, o, true);
                const float4 pbl = shfl_f4(bl, o, false), pbh = shfl_f4(bh, o, false);
                if (lane >= o) {
                    a = min(a, pa);
                    box_union(al, ah, pal, pah);
                }
                if (lane + o < RW) {
                    b = min(b, pb);
                    box_union(bl, bh, pbl, pbh);
                }
            }
            // exclusive: the inclusive value of the neighbour (identity at the ends)
            const int ea = __shfl_up_sync(0xffffffffu, a, 1), eb = __shfl_down_sync(0xffffffffu, b, 1);
            const float4 eal = shfl_f4(al, 1, true), eah = shfl_f4(ah, 1, true);
            const float4 ebl = shfl_f4(bl, 1, false), ebh = shfl_f4(bh, 1, false);
            if (in) {
                S.xpm[lane] = lane > 0 ? ea : BIG_DELTA;
                S.xsm[lane] = lane + 1 < RW ? eb : BIG_DELTA;
                S.xplo[lane] = lane > 0 ? eal : ident_lo();
                S.xphi[lane] = lane > 0 ? eah : ident_hi();
                S.xslo[lane] = lane + 1 < RW ? ebl : ident_lo();
                S.xshi[lane] = lane + 1 < RW ? ebh : ident_hi();
            }
        }
        __syncthreads();
        const int wpm = S.xpm[warp], wsm = S.xsm[warp];
        // strict prefix (suffix) minimum: delta below every delta to its left (right)
        // in the chunk
        const int ppm = __shfl_up_sync(0xffffffffu, pm, 1), nsm = __shfl_down_sync(0xffffffffu, sm, 1);
        const int epm = min(wpm, lane > 0 ? ppm : BIG_DELTA);
        const int esm = min(wsm, lane < 31 ? nsm : BIG_DELTA);
        const bool pre = dk < epm, suf = dk < esm;
        // the chunk's leaves up to leaf j, and after it
        float4 up_lo = S.xplo[warp], up_hi = S.xphi[warp];
        box_union(up_lo, up_hi, plo, phi);
        float4 af_lo = S.xslo[warp], af_hi = S.xshi[warp];
        {
            const float4 nl = shfl_f4(slo, 1, false), nh = shfl_f4(shi, 1, false);
            if (lane < 31) box_union(af_lo, af_hi, nl, nh);
        }
        // node of boundary j spans chunks: no smaller delta on one side inside the chunk,
        // or j is the boundary to the next chunk
        const bool span = j <= n - 2 && (j == c1 - 1 || (S.flag[tid] != 3u));
        const unsigned bs = __ballot_sync(0xffffffffu, suf), bp = __ballot_sync(0xffffffffu, pre);
        const unsigned bt = __ballot_sync(0xffffffffu, span);
        if (lane == 0) {
            S.wsr[warp] = __popc(bs);
            S.wpr[warp] = __popc(bp);
            S.wtop[warp] = __popc(bt);
        }
        __syncthreads();
        if (warp == 0) {  // counts over the warps before / after warp `lane`, and in all
            const bool in = lane < RW;
            const int vs = in ? S.wsr[lane] : 0, vp = in ? S.wpr[lane] : 0, vt = in ? S.wtop[lane] : 0;
            int is = vs, ip = vp, it = vt;  // inclusive prefix sums
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int qs = __shfl_up_sync(0xffffffffu, is, o), qp = __shfl_up_sync(0xffffffffu, ip, o);
                const int qt = __shfl_up_sync(0xffffffffu, it, o);
                if (lane >= o) {
                    is += qs;
                    ip += qp;
                    it += qt;
                }
            }
            const int ts = __shfl_sync(0xffffffffu, is, 31), tp = __shfl_sync(0xffffffffu, ip, 31);
            const int tt = __shfl_sync(0xffffffffu, it, 31);
            if (in) {
                S.xos[lane] = ts - is;  // suffix records after warp `lane`
                S.xop[lane] = ip - vp;
                S.xot[lane] = it - vt;
            }
            if (lane == 0) {
                S.nrec[0] = ts;
                S.nrec[1] = tp;
                S.nrec[2] = tt;
            }
        }
        __syncthreads();
        const int os = __popc(bs & ~((2u << lane) - 1u)) + S.xos[warp];
        const int op = __popc(bp & ((1u << lane) - 1u)) + S.xop[warp];
        const int ot = __popc(bt & ((1u << lane) - 1u)) + S.xot[warp];
        if (suf && os < 32) {
            cv.srec[32 * chunk + os] = make_int2(j, dk);
            cv.sbox[2 * (32 * chunk + os)] = af_lo;
            cv.sbox[2 * (32 * chunk + os) + 1] = af_hi;
        }
        if (pre && op < 32) {
            cv.prec[32 * chunk + op] = make_int2(j, dk);
            cv.pbox[2 * (32 * chunk + op)] = up_lo;
            cv.pbox[2 * (32 * chunk + op) + 1] = up_hi;
        }
        if (tid == BUILD_LEAVES - 1) {  // holds the whole chunk's prefix
            cv.rcnt[3 * chunk] = min(S.nrec[0], 32);
            cv.rcnt[3 * chunk + 1] = min(S.nrec[1], 32);
            cv.rcnt[3 * chunk + 2] = min(S.nrec[2], 64);
            cv.cmin[chunk] = min(wpm, pm);
            cv.cbox[2 * chunk] = up_lo;
            cv.cbox[2 * chunk + 1] = up_hi;
        }
        if (span && ot < 64) cv.top[64 * chunk + ot] = make_int2(j, dk);  // at most 61 per chunk
    }
    __syncthreads();  // the shared arrays are reused by the CTA's next chunk
}

// After chunk c's summary: the summaries per 32, 1024 and 32768 chunks.  Each entry
// of level v counts its members as they finish (the CTA fences its writes, then
// counts); the CTA that brings the count to the group's size reduces the group
// into the level-v entry and counts that entry into level v + 1.
__device__ void level_up(const RebuildArgs& A, int c, int n, int* s_last) {
    const ChunkView& cv = A.cv;
    const int lane = threadIdx.x & 31;
    int cnt[NLEV];
    level_counts(n, cnt);
    int e = c;  // the finished entry of level v - 1
    for (int v = 1; v < NLEV; ++v) {
        const int grp = e >> 5;
        __threadfence();  // every thread's summary writes before the count
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t members = (uint32_t)min(32, cnt[v - 1] - 32 * grp);
            *s_last = atomicAdd(A.gdone + cv.lev_off[v] + grp, 1u) == members - 1u ? 1 : 0;
            __threadfence();  // the other members' writes before this CTA's reads
        }
        __syncthreads();
        const bool last = *s_last != 0;
        __syncthreads();  // s_last is rewritten on the next level
        if (!last) return;
        if (threadIdx.x < 32) {
            const int k = 32 * grp + lane;
            int m = BIG_DELTA;
            float4 blo = ident_lo(), bhi = ident_hi();
            if (k < cnt[v - 1]) {
                m = __ldcg(cv.cmin + cv.lev_off[v - 1] + k);
                blo = __ldcg(cv.cbox + 2 * (cv.lev_off[v - 1] + k));
                bhi = __ldcg(cv.cbox + 2 * (cv.lev_off[v - 1] + k) + 1);
            }
            warp_box_reduce(blo, bhi);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) {
                cv.cmin[cv.lev_off[v] + grp] = m;
                cv.cbox[2 * (cv.lev_off[v] + grp)] = blo;
                cv.cbox[2 * (cv.lev_off[v] + grp) + 1] = bhi;
            }
        }
        e = grp;
    }
}

// Nearest entry of level 0 (a chunk) left of chunk c (right, with right) whose min
// delta is below d, through the summary levels: scan the 32 entries of the current
// group, climb a level while nothing qualifies, then descend into the first group
// that does.  -1: none.
__device__ int nearest_chunk(const ChunkView& cv, const int cnt[NLEV], int c, int d, bool right, int lane, int* err) {
    int idx = c;
    for (int v = 0; v < NLEV; ++v) {
        const int* m = cv.cmin + cv.lev_off[v];
        const int base = idx & ~31, e = base + lane;
        const bool hit = (right ? e > idx : e < idx) && e < cnt[v] && __ldcg(m + e) < d;
        unsigned b = __ballot_sync(0xffffffffu, hit);
        if (b) {
            int f = right ? base + __ffs(b) - 1 : base + 31 - __clz(b);
            for (int u = v - 1; u >= 0; --u) {  // descend: the first qualifying entry of group f
                const int b2 = 32 * f, e2 = b2 + lane;
                const bool h2 = e2 < cnt[u] && __ldcg(cv.cmin + cv.lev_off[u] + e2) < d;
                b = __ballot_sync(0xffffffffu, h2);
                if (!b) {  // the group's min said otherwise: corrupt summaries
                    if (lane == 0) atomicOr(err, ERR_TIMEOUT);
                    return -1;
                }
                f = right ? b2 + __ffs(b) - 1 : b2 + 31 - __clz(b);
            }
            return f;
        }
        if (right ? base + 32 >= cnt[v] : base == 0) return -1;  // no group beyond this one
        idx >>= 5;
    }
    return -1;
}

// First record (in the records' order) of chunk c with delta below d whose position is
// left of g (right of g, with right); g < 0: any position.  -1: none.
__device__ __forceinline__ int first_record(const int2* rec, int count, int g, int d, bool right, int lane,
                                            int2& out) {
    const int2 q = lane < count ? __ldcg(rec + lane) : make_int2(0, BIG_DELTA);
    const bool hit = lane < count && q.y < d && (g < 0 || (right ? q.x > g : q.x < g));
    const unsigned b = __ballot_sync(0xffffffffu, hit);
    if (!b) return -1;
    const int k = __ffs(b) - 1;
    out = make_int2(__shfl_sync(0xffffffffu, q.x, k), __shfl_sync(0xffffffffu, q.y, k));
    return k;
}

// union of the leaf boxes of chunks [a, b] (warp-uniform a, b), in every lane
__device__ void chunk_union(const ChunkView& cv, const int cnt[NLEV], int a, int b, int lane, float4& lo,
                            float4& hi) {
    float4 ul = ident_lo(), uh = ident_hi();
    for (int v = 0; v < NLEV && a <= b; ++v) {
        const float4* bx = cv.cbox + 2 * cv.lev_off[v];
        if ((a >> 5) == (b >> 5) || v == NLEV - 1) {
            for (int e = a + lane; e <= b; e += 32) box_union(ul, uh, __ldcg(bx + 2 * e), __ldcg(bx + 2 * e + 1));
            break;
        }
        const int e1 = a + lane, e2 = (b & ~31) + lane;
        if (e1 <= (a | 31)) box_union(ul, uh, __ldcg(bx + 2 * e1), __ldcg(bx + 2 * e1 + 1));
        if (e2 <= b) box_union(ul, uh, __ldcg(bx + 2 * e2), __ldcg(bx + 2 * e2 + 1));
        a = (a >> 5) + 1;
        b = (b >> 5) - 1;
    }
    warp_box_reduce(ul, uh);
    box_union(lo, hi, ul, uh);
}

// The nodes whose leaf range spans chunks, one warp each, independently: the range
// ends are the nearest boundaries with a smaller delta on either side (the first
// suffix / prefix record past the node with a smaller delta, in the node's chunk or
// in the nearest chunk with a smaller min), the box is the union of the leaf boxes in
// the range (the records' partial unions and whole chunks between), and the node
// enters its parent (the range end with the larger delta) as the climb would have
// put it there.
__device__ void phase_top(const RebuildArgs& A, int n) {
    const ChunkView& cv = A.cv;
    int cnt[NLEV];
    level_counts(n, cnt);
    const int lane = (int)(threadIdx.x & 31u);
    // each chunk's nodes that span chunks sit in its 64 slots; iteration `it` takes slot
    // it / F of chunk it % F, so the (few, low) occupied slots spread over all warps
    const uint32_t F = (uint32_t)cnt[0], slots = 64u * F;
    const uint32_t nw = gridDim.x * RW;
    for (uint32_t it = blockIdx.x * RW + (threadIdx.x >> 5); it < slots; it += nw) {
        const uint32_t ch = it % F, sl = it / F;
        if ((int)sl >= __ldcg(cv.rcnt + 3 * ch + 2)) continue;
        const int2 item = __ldcg(cv.top + 64 * ch + sl);
        const int g = item.x, d = item.y, c = g / BUILD_LEAVES;
        if (g < 0 || g > n - 2 || c >= cnt[0]) {
            if (lane == 0) atomicOr(A.err, ERR_TIMEOUT);
            continue;
        }
        // left end: boundary jl (leaves from jl + 1), -1 = none
        int2 q;
        int jl = -1, dlft = -1, cl = -1;
        float4 lo = ident_lo(), hi = ident_hi();
        int k = first_record(cv.srec + 32 * c, __ldcg(cv.rcnt + 3 * c), g, d, false, lane, q);
        int cc = c;
        if (k < 0) {
            cc = nearest_chunk(cv, cnt, c, d, false, lane, A.err);
            if (cc >= 0) k = first_record(cv.srec + 32 * cc, __ldcg(cv.rcnt + 3 * cc), -1, d, false, lane, q);
        }
        if (k >= 0) {
            jl = q.x;
            dlft = q.y;
            cl = cc;
            box_union(lo, hi, __ldcg(cv.sbox + 2 * (32 * cc + k)), __ldcg(cv.sbox + 2 * (32 * cc + k) + 1));
        }
        // right end: boundary jr (leaves up to jr), n - 1 = none
        int jr = n - 1, drgt = -1, cr = cnt[0] - 1;
        k = first_record(cv.prec + 32 * c, __ldcg(cv.rcnt + 3 * c + 1), g, d, true, lane, q);
        cc = c;
        if (k < 0) {
            cc = nearest_chunk(cv, cnt, c, d, true, lane, A.err);
            if (cc >= 0) k = first_record(cv.prec + 32 * cc, __ldcg(cv.rcnt + 3 * cc + 1), -1, d, true, lane, q);
        }
        if (k >= 0) {
            jr = q.x;
            drgt = q.y;
            cr = cc;
            box_union(lo, hi, __ldcg(cv.pbox + 2 * (32 * cc + k)), __ldcg(cv.pbox + 2 * (32 * cc + k) + 1));
        } else {
            box_union(lo, hi, __ldcg(cv.cbox + 2 * cr), __ldcg(cv.cbox + 2 * cr + 1));  // the last chunk
        }
        chunk_union(cv, cnt, cl + 1, cr - 1, lane, lo, hi);
        if (lane == 0) {
            if (jl < 0 && jr == n - 1) {
                A.root->root = g;
                A.root->top_lo = lo;
                A.root->top_hi = hi;
            } else {
                const bool is_a = drgt > dlft;
                write_side(A.nodes, A.range, is_a ? jr : jl, is_a, lo, hi, g, jl + 1, jr, is_a ? dlft : drgt);
            }
        }
    }
}

// ---- the launch -----------------------------------------------------------------------------------
__global__ void __launch_bounds__(RB, 2) k_rebuild(const RebuildArgs A) {
    extern __shared__ __align__(16) unsigned char rb_smem[];
    __shared__ uint32_t s_scan[32];
    __shared__ float s_red[6 * RW];
    __shared__ float s_frame[8];
    __shared__ int s_ok, s_claim;
    uint32_t target = 0;
    const int nt = A.nt;
    // the last build's sorted list (keys[cur], vals[cur]) and codes are usable: read
    // before any CTA can change the root record
    const bool coherent = A.coherent && ld_volatile(reinterpret_cast<const uint32_t*>(&A.root->perm_valid)) != 0u;
    const int cur = coherent ? (int)ld_volatile(reinterpret_cast<const uint32_t*>(&A.root->sorted)) & 1 : 1;
    const int n_prev = A.root->n_leaves;
    // what the later phases need at zero (read only after the next barrier)
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        A.chg[0] = 0u;
        A.root->n_tris = nt;
    }
    {
        const size_t zw = (size_t)PASSES * RADIX + (size_t)PASSES * A.tiles_sort * RADIX + PASSES;
        for (size_t k = (size_t)blockIdx.x * RB + threadIdx.x; k < zw; k += (size_t)gridDim.x * RB) A.ghist[k] = 0u;
        for (int k = blockIdx.x * RB + threadIdx.x; k < A.n_entries; k += gridDim.x * RB) A.gdone[k] = 0u;
    }
    phase_verts(A);
    bool ok = grid_barrier(A.sync, target, true, A.err, &s_ok);
    if (ok) phase_boxes(A, s_red);
    ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
    if (ok) phase_codes(A, coherent, s_red, s_frame);
    ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
    // the sort: same decision in every CTA (from words complete at the barrier)
    const uint32_t nchg = ld_volatile(A.chg);
    const bool merge = coherent && nchg <= (uint32_t)CHG_CAP;
    int after = cur;  // buffer holding this build's sorted list
    bool fresh = true;  // the sorted list changed: de-duplicate it again
    if (merge) {
        if (nchg == 0u) {
            fresh = false;  // every code as before: the last build's list and leaves stand
        } else {
            after = cur ^ 1;
            if (ok)
                phase_merge(A, (int)nchg, A.keys[cur], A.vals[cur], A.keys[after], A.vals[after],
                            *reinterpret_cast<MergeSmem*>(rb_smem));
            ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
        }
    } else {
        if (ok) phase_hist(A, reinterpret_cast<uint32_t*>(rb_smem));
        ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
        for (int p = 0; p < PASSES; ++p) {
            if (ok) phase_sort_pass(A, p, *reinterpret_cast<SortSmem*>(rb_smem), s_scan, &s_claim);
            ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
        }
        after = (PASSES - 1) & 1;
    }
    int n = n_prev;
    if (fresh) {
        if (ok) phase_unique_count(A, A.keys[after], s_scan);
        ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
        if (ok) n = phase_unique_write(A, A.keys[after], A.vals[after], s_scan);
        ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // the sort buffers now hold this build's list, unless some wait gave up
        const bool bad = !ok || (ld_volatile(reinterpret_cast<const uint32_t*>(A.err)) & ERR_TIMEOUT) != 0u;
        A.root->perm_valid = bad ? 0 : 1;
        A.root->sorted = after;
    }
    n = min(n, nt);
    const int chunks = (n + BUILD_LEAVES - 1) / BUILD_LEAVES;
    if (ok)
        for (int c = blockIdx.x; c < chunks; c += gridDim.x) {
            build_chunk(A, c, n, *reinterpret_cast<BuildSmem*>(rb_smem));
            level_up(A, c, n, &s_claim);
        }
    ok = grid_barrier(A.sync, target, ok, A.err, &s_ok);
    if (ok) phase_top(A, n);
    // the last CTA out leaves both counters at zero for the next launch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(A.sync + 1, 1u) == gridDim.x - 1u) {
            atomicExch(A.sync, 0u);
            atomicExch(A.sync + 1, 0u);
        }
    }
}

// Self-test of the grid barrier's bounded wait: one CTA waits for an arrival count
// that no other CTA will bring; the wait gives up after kGridWaitNs, records
// ERR_TIMEOUT and returns.
__global__ void k_selftest_grid_wait(uint32_t* ctr, int* err) {
    __shared__ int s_ok;
    uint32_t target = 1;  // as if one barrier of this one-CTA launch had passed
    (void)grid_barrier(ctr, target, true, err, &s_ok);
}

// Self-test of the look-back's bounded wait: one thread looks back from tile 1 at a
// status word (tile 0's) that nothing publishes; the walk gives up after SPIN_LIMIT
// sleeps, records ERR_TIMEOUT and returns.
__global__ void k_selftest_look_back(const uint32_t* status, int* err) {
    if (threadIdx.x == 0) (void)look_back(status, 1, 1, err);
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// CTAs of k_rebuild that fit on the device at once (cooperative launch limit)
int resident_ctas() {
    static std::mutex mu;
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!cached[dev]) {
        int sms = 0, per = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rebuild, RB, kSmemBytes) != cudaSuccess) return 0;
        cached[dev] = sms * per;
    }
    return cached[dev];
}

}  // namespace

void BvhBuffers::plan(Arena& a, int nv_, int nt_, bool normals) {
    nv = nv_;
    nt = nt_;
    has_normals = normals;
    tiles_sort = nt > 0 ? cdiv(nt, SORT_TILE) : 0;
    max_ctas = std::max(1, cdiv(std::max(nt, 1), RB));
    int ni = nt > 1 ? nt - 1 : 1;
    a.want(&xyz_in, (size_t)nv * 3 + 4);
    a.want(&nrm_in, (size_t)nv * 3 + 4);
    a.want(&verts, (size_t)nv + 1);
    a.want(&tris, (size_t)nt * 3 + 4);
    a.want(&tri_box, (size_t)nt * 2 + 2);
    a.want(&tri_leaf, (size_t)nt * 2 + 2);
    a.want(&codes, (size_t)nt + 1);
    for (int k = 0; k < 2; ++k) {
        a.want(&keys[k], (size_t)nt + 1);
        a.want(&vals[k], (size_t)nt + 1);
    }
    a.want(&ucode, (size_t)nt + 1);
    a.want(&utri, (size_t)nt + 1);
    a.want(&nodes, (size_t)ni);
    a.want(&leaves, (size_t)nt * 2 + 2);
    a.want(&range, (size_t)ni);
    chunks = cdiv(std::max(nt, 1), BUILD_LEAVES);
    int entries = 0, e = chunks;
    for (int v = 0; v < NLEV; ++v) {
        lev_off[v] = entries;
        entries += e;
        e = cdiv(e, 32);
    }
    a.want(&cmin, (size_t)entries);
    a.want(&cbox, 2 * (size_t)entries);
    a.want(&srec, 32 * (size_t)chunks);
    a.want(&sbox, 64 * (size_t)chunks);
    a.want(&prec, 32 * (size_t)chunks);
    a.want(&pbox, 64 * (size_t)chunks);
    a.want(&rcnt, 3 * (size_t)chunks);
    a.want(&top, 64 * (size_t)chunks);
    a.want(&root, 1);
    // histograms | sort status (PASSES x tiles x RADIX) | sort counters (the launch
    // clears them) | CTA box unions | CTA leaf counts | change list | barrier counters
    scratch_words = (size_t)PASSES * RADIX + (size_t)PASSES * tiles_sort * RADIX + PASSES;
    a.want(&scratch, scratch_words);
    a.want(&part, 8 * (size_t)max_ctas);
    a.want(&ucnt, (size_t)max_ctas);
    a.want(&chg, 1 + 3 * (size_t)CHG_CAP);
    a.want(&sync, 2);
    n_entries = entries;
    a.want(&gdone, (size_t)entries);
}

cudaError_t lbvh_build(BvhBuffers& b, float thickness, float box_depth, int* d_err, cudaStream_t s, const float* xyz,
                       const float* nrm, float4* margin_state, int64_t m0, int64_t m1) {
    if (b.nt == 0) return cudaSuccess;
    const int res = resident_ctas();
    if (res <= 0) return cudaErrorLaunchOutOfResources;
    RebuildArgs A;
    A.xyz = xyz ? xyz : b.xyz_in;
    A.nrm = b.has_normals ? (xyz ? nrm : b.nrm_in) : nullptr;
    A.margin_state = margin_state;
    A.m0 = m0;
    A.m1 = m1;
    A.tris = b.tris;
    A.nv = b.nv;
    A.nt = b.nt;
    A.thickness = thickness;
    A.depth = box_depth;
    A.coherent = b.coherent ? 1 : 0;
    A.tiles_sort = b.tiles_sort;
    A.verts = b.verts;
    A.tri_box = b.tri_box;
    A.tri_leaf = b.tri_leaf;
    A.codes = b.codes;
    for (int k = 0; k < 2; ++k) {
        A.keys[k] = b.keys[k];
        A.vals[k] = b.vals[k];
    }
    A.ucode = b.ucode;
    A.utri = b.utri;
    A.nodes = b.nodes;
    A.leaves = b.leaves;
    A.range = b.range;
    A.root = b.root;
    A.cv = ChunkView{b.cmin, b.cbox, b.srec, b.sbox, b.prec, b.pbox, b.rcnt, b.top,
                     {b.lev_off[0], b.lev_off[1], b.lev_off[2], b.lev_off[3]}};
    A.ghist = b.scratch;
    A.sstat = A.ghist + PASSES * RADIX;
    A.scount = A.sstat + (size_t)PASSES * b.tiles_sort * RADIX;
    A.part = b.part;
    A.ucnt = b.ucnt;
    A.chg = b.chg;
    A.sync = b.sync;
    A.gdone = b.gdone;
    A.n_entries = b.n_entries;
    A.err = d_err;
    const int grid = std::min(res, b.max_ctas);
    void* args[] = {&A};
    return cudaLaunchCooperativeKernel((const void*)k_rebuild, dim3(grid), dim3(RB), args, kSmemBytes, s);
}

cudaError_t launch_selftest_look_back(const uint32_t* zero_status, int* err, cudaStream_t s) {
    k_selftest_look_back<<<1, 32, 0, s>>>(zero_status, err);
    return cudaGetLastError();
}

cudaError_t launch_selftest_grid_wait(uint32_t* zero_counter, int* err, cudaStream_t s) {
    k_selftest_grid_wait<<<1, 32, 0, s>>>(zero_counter, err);
    return cudaGetLastError();
}

}  // namespace visg
