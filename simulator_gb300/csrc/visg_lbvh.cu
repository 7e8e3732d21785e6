// visg_lbvh.cu — per-step body LBVH build on the device.
//
// Reference (BVHAccel, src/bvh/bvh.cu:154-297; cudaBRT.cu:9-206) builds once per
// body with a device->host->device round trip: expanded boxes and Morton codes on
// the GPU, std::sort + duplicate removal on the CPU, then Karras internal nodes and
// an atomic-counter refit on the GPU.  Here the whole build stays on the device,
// in up to ten stream-ordered kernels, so it can run every step and be captured in a
// CUDA graph:
//   k_body_prep   vertex_extend (Mesh.cpp:101-117): v += thickness * n
//   k_tri_boxes   expanded triangle boxes (primitive.cu:79-91) + the Morton frame
//                 (identity box U all boxes) by warp-shuffle min/max reduction
//   k_morton      Morton code of each box centroid in the frame (bvh.cu:20-41,71-79;
//                 bbox.h:97-127) + the digit histograms of all four radix passes
//   k_coherence   (bodies rebuilt every step) is the last build's permutation still
//                 the stable order of the new codes?  Then the radix passes exit at
//                 once; if every code is unchanged too, so does k_unique
//   k_sort_pass   x4: stable LSD radix pass, 8-bit digits, decoupled look-back
//                 (ties keep triangle order, i.e. sort by (code, triangle))
//   k_unique      keep the first triangle of every distinct code
//                 (remove_redundant, Utilities.h:35-55), look-back compaction
//   k_build       bottom-up radix-tree build fused with the refit, per chunk of 512
//                 sorted leaves: each leaf thread climbs with handshakes in shared
//                 memory while both children lie in the chunk; the parent of range
//                 [l, r] is the boundary with the longer common prefix (delta(l-1,l)
//                 vs delta(r,r+1), delta = clz(a ^ b) as cudaBRT.cu:9-19), the second
//                 child to arrive merges both boxes into the identity box
//                 (calculateBoudingBox, cudaBRT.cu:166-206) and continues.  Each chunk
//                 then publishes a summary for the nodes that span chunks
//   k_build_top   one warp per node that spans chunks: its range ends are the nearest
//                 boundaries with a smaller delta, its box the union of its leaves'
//                 boxes, both read off the chunk summaries
//                 Nodes are numbered by their split position; the tree is the same
//                 binary radix tree processInternalNode (cudaBRT.cu:120-161) builds,
//                 and visg_export_lbvh renumbers it into the reference's layout.
// Every wait is bounded; a wait that gives up sets ERR_TIMEOUT and the host reports
// VISG_ERR_TIMEOUT.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "visg_internal.cuh"

namespace visg {

namespace {

constexpr int BUILD_THREADS = 256;
constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;  // 2048
constexpr int RADIX = 256;
constexpr int PASSES = 4;
static_assert(PASSES % 2 == 0, "the last pass writes keys[1] / vals[1], which k_coherence reads");
constexpr uint32_t ST_AGG = 1u << 30;
constexpr uint32_t ST_PREFIX = 2u << 30;
constexpr uint32_t ST_VALUE = (1u << 30) - 1u;
constexpr int SPIN_LIMIT = 1 << 22;
// rebuild mode word (zero before every build): what k_coherence found
constexpr uint32_t M_RAN = 1u;       // the check ran (else every pass does its work)
constexpr uint32_t M_UNSORTED = 2u;  // the last permutation does not sort the new codes
constexpr uint32_t M_CHANGED = 4u;   // some code changed
__device__ __forceinline__ bool skip_sort(uint32_t m) { return (m & M_RAN) && !(m & M_UNSORTED); }
__device__ __forceinline__ bool skip_unique(uint32_t m) { return (m & M_RAN) && !(m & (M_UNSORTED | M_CHANGED)); }

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) { *reinterpret_cast<volatile uint32_t*>(p) = v; }

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

// inclusive scan of one value per thread over a 256-thread block
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
        uint32_t w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t r = v + (warp > 0 ? s_warp[warp - 1] : 0u);
    __syncthreads();
    return r;
}

// ------------------------------------------------------------------------------------------
__global__ void k_body_prep(const float* __restrict__ xyz, const float* __restrict__ nrm, int nv, float thickness,
                            float4* __restrict__ verts, BvhRoot* root, int nt) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v == 0) {
        root->acc[0] = root->acc[1] = root->acc[2] = f2ord(100.0f);   // identity box min (bbox.h:17-22)
        root->acc[3] = root->acc[4] = root->acc[5] = f2ord(-100.0f);  // identity box max
        root->n_tris = nt;
    }
    if (v >= nv) return;
    float x = xyz[3 * v], y = xyz[3 * v + 1], z = xyz[3 * v + 2];
    if (nrm) {
        x = __fadd_rn(x, __fmul_rn(thickness, nrm[3 * v]));
        y = __fadd_rn(y, __fmul_rn(thickness, nrm[3 * v + 1]));
        z = __fadd_rn(z, __fmul_rn(thickness, nrm[3 * v + 2]));
    }
    verts[v] = make_float4(x, y, z, 0.0f);
}

__device__ __forceinline__ void box_add(f3& lo, f3& hi, f3 p) {
    lo.x = fminf(lo.x, p.x); lo.y = fminf(lo.y, p.y); lo.z = fminf(lo.z, p.z);
    hi.x = fmaxf(hi.x, p.x); hi.y = fmaxf(hi.y, p.y); hi.z = fmaxf(hi.z, p.z);
}

__global__ void __launch_bounds__(BUILD_THREADS)
k_tri_boxes(const float4* __restrict__ verts, int nv, const uint32_t* __restrict__ tris, int nt, float depth,
            float4* __restrict__ tri_box, float4* __restrict__ tri_leaf, BvhRoot* root, int* err) {
    __shared__ float s_red[6][BUILD_THREADS / 32];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    f3 lo = mk3(100.0f, 100.0f, 100.0f), hi = mk3(-100.0f, -100.0f, -100.0f);
    if (t < nt) {
        // vertex indices come from the caller: one out of range is recorded and read
        // as vertex 0, so no load leaves the vertex array (the build's result is then
        // reported as failed)
        uint32_t i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
        if (i0 >= (uint32_t)nv || i1 >= (uint32_t)nv || i2 >= (uint32_t)nv) {
            atomicOr(err, ERR_INDEX);
            i0 = i0 < (uint32_t)nv ? i0 : 0u;
            i1 = i1 < (uint32_t)nv ? i1 : 0u;
            i2 = i2 < (uint32_t)nv ? i2 : 0u;
        }
        f3 v0 = xyz(__ldg(&verts[i0]));
        f3 v1 = xyz(__ldg(&verts[i1]));
        f3 v2 = xyz(__ldg(&verts[i2]));
        f3 n = normalize(cross(sub(v1, v0), sub(v2, v0)));  // Primitive::d_get_normal
        f3 blo = v0, bhi = v0;                                 // BBox(v0).expand(v1).expand(v2)
        box_add(blo, bhi, v1);
        box_add(blo, bhi, v2);
        f3 dn = mul(depth, n);
        box_add(blo, bhi, sub(v0, dn));
        box_add(blo, bhi, sub(v1, dn));
        box_add(blo, bhi, sub(v2, dn));
        tri_box[2 * t] = make_float4(blo.x, blo.y, blo.z, 0.0f);
        tri_box[2 * t + 1] = make_float4(bhi.x, bhi.y, bhi.z, 0.0f);
        tri_leaf[2 * t] = make_float4(v0.x, v0.y, v0.z, n.x);
        tri_leaf[2 * t + 1] = make_float4(n.y, n.z, __int_as_float(t), 0.0f);
        lo = blo;
        hi = bhi;
    }
    // frame = identity U every box: block min/max, then one ordered atomic per block
    float r[6] = {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = fminf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
#pragma unroll
        for (int k = 3; k < 6; ++k) r[k] = fmaxf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 6; ++k) s_red[k][warp] = r[k];
    __syncthreads();
    if (threadIdx.x < 6) {
        int k = threadIdx.x;
        float v = s_red[k][0];
        for (int w = 1; w < BUILD_THREADS / 32; ++w) v = k < 3 ? fminf(v, s_red[k][w]) : fmaxf(v, s_red[k][w]);
        if (k < 3) atomicMin(&root->acc[k], f2ord(v));
        else atomicMax(&root->acc[k], f2ord(v));
    }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {  // bvh.cu:20-27
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void __launch_bounds__(BUILD_THREADS)
k_morton(const float4* __restrict__ tri_box, int nt, BvhRoot* root, uint32_t* __restrict__ codes,
         uint32_t* __restrict__ ghist /* PASSES*RADIX */) {
    __shared__ uint32_t s_hist[PASSES][RADIX];
    __shared__ float s_frame[6];
    for (int k = threadIdx.x; k < PASSES * RADIX; k += blockDim.x) (&s_hist[0][0])[k] = 0;
    if (threadIdx.x < 6) s_frame[threadIdx.x] = ord2f(root->acc[threadIdx.x]);
    __syncthreads();
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        root->frame_lo = make_float4(s_frame[0], s_frame[1], s_frame[2], 0.0f);
        root->frame_hi = make_float4(s_frame[3], s_frame[4], s_frame[5], 0.0f);
    }
    uint32_t code = 0u;
    if (t < nt) {
        float4 lo = tri_box[2 * t], hi = tri_box[2 * t + 1];
        f3 c = divs(add(xyz(lo), xyz(hi)), 2.0f);  // BBox::centroid
        f3 fmn = mk3(s_frame[0], s_frame[1], s_frame[2]);
        f3 ext = sub(mk3(s_frame[3], s_frame[4], s_frame[5]), fmn);
        f3 q = mk3(0.0f, 0.0f, 0.0f);
        if (length(ext) != 0.0f) q = divv(sub(c, fmn), ext);  // BBox::getUnitcubePosOf
        float x = fminf(fmaxf(__fmul_rn(q.x, 1024.0f), 0.0f), 1023.0f);
        float y = fminf(fmaxf(__fmul_rn(q.y, 1024.0f), 0.0f), 1023.0f);
        float z = fminf(fmaxf(__fmul_rn(q.z, 1024.0f), 0.0f), 1023.0f);
        code = expand_bits((uint32_t)x) * 4u + expand_bits((uint32_t)y) * 2u + expand_bits((uint32_t)z);
        codes[t] = code;
    }
    // digit counts of the four radix passes; the two high digits are nearly constant
    // across a block's neighbouring triangles, so their lanes add once per equal digit
    const int lane = threadIdx.x & 31;
    const bool ok = t < nt;
#pragma unroll
    for (int p = 0; p < PASSES; ++p) {
        const uint32_t dig = (code >> (8 * p)) & 255u;
        if (p < 2) {
            if (ok) atomicAdd(&s_hist[p][dig], 1u);
        } else {
            const uint32_t peers = __match_any_sync(0xffffffffu, ok ? dig : RADIX);
            if (ok && lane == __ffs(peers) - 1) atomicAdd(&s_hist[p][dig], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < PASSES * RADIX; k += blockDim.x) {
        uint32_t v = (&s_hist[0][0])[k];
        if (v) atomicAdd(&ghist[k], v);
    }
}

// Temporal coherence of a rebuild.  keys1/vals1 hold the last build's sorted codes
// and permutation (when root->perm_valid).  The stable sort of the new codes by
// (code, triangle) is unique, so if the last permutation orders them (non-decreasing
// codes, equal codes by increasing triangle), it is that sort: keys1 takes the new
// codes in that order and the radix passes have nothing to do.  If no code changed,
// the de-duplicated leaves are the last build's too.
__global__ void __launch_bounds__(BUILD_THREADS)
k_coherence(const uint32_t* __restrict__ codes, uint32_t* keys1, const uint32_t* __restrict__ vals1, int nt,
            const BvhRoot* __restrict__ root, uint32_t* mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t bad = 0;
    if (!root->perm_valid) {
        bad = M_UNSORTED | M_CHANGED;
    } else if (i < nt) {
        const uint32_t p = vals1[i];
        if (p >= (uint32_t)nt) {
            bad = M_UNSORTED | M_CHANGED;
        } else {
            const uint32_t c = codes[p];
            if (c != keys1[i]) bad |= M_CHANGED;
            if (i > 0) {
                const uint32_t q = vals1[i - 1];
                const uint32_t cq = q < (uint32_t)nt ? codes[q] : 0xffffffffu;
                if (q >= (uint32_t)nt || cq > c || (cq == c && q > p)) bad |= M_UNSORTED;
            }
            keys1[i] = c;  // only this thread reads or writes entry i
        }
    }
    bad = __reduce_or_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && bad) atomicOr(mode, bad);
    if (i == 0) atomicOr(mode, M_RAN);
}

// One stable LSD pass over 8-bit digit (key >> shift) & 255.  Tiles are claimed in
// launch order through an atomic counter, so every tile a block waits on belongs to a
// block that is already running: the look-back always terminates.
__global__ void __launch_bounds__(SORT_THREADS)
k_sort_pass(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
            uint32_t* __restrict__ vout, int n, int shift, const uint32_t* __restrict__ ghist,
            uint32_t* status, uint32_t* counter, const uint32_t* __restrict__ mode, int* err) {
    if (skip_sort(*mode)) return;  // the last build's order stands
    __shared__ uint32_t s_whist[SORT_THREADS / 32][RADIX + 1];
    __shared__ uint32_t s_tstart[RADIX];
    __shared__ uint32_t s_gbase[RADIX];
    __shared__ uint32_t s_keys[SORT_TILE];
    __shared__ uint32_t s_vals[SORT_TILE];
    __shared__ uint32_t s_warp[32];
    __shared__ int s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = (int)atomicAdd(counter, 1u);
    for (int k = tid; k < (SORT_THREADS / 32) * (RADIX + 1); k += SORT_THREADS) (&s_whist[0][0])[k] = 0;
    __syncthreads();
    const int tile = s_tile;
    const int base = tile * SORT_TILE + warp * (32 * SORT_ITEMS);
    uint32_t key[SORT_ITEMS], val[SORT_ITEMS], rank[SORT_ITEMS];
    int dig[SORT_ITEMS];
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        int idx = base + j * 32 + lane;  // warp-striped: j-major order is input order
        if (idx < n) {
            key[j] = kin[idx];
            val[j] = vin ? vin[idx] : (uint32_t)idx;
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
        uint32_t peers = __match_any_sync(0xffffffffu, dig[j]);
        int leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (lane == leader) {
            before = s_whist[warp][dig[j]];
            s_whist[warp][dig[j]] = before + __popc(peers);
        }
        before = __shfl_sync(0xffffffffu, before, leader);
        rank[j] = before + __popc(peers & ((1u << lane) - 1u));
        __syncwarp();
    }
    __syncthreads();
    // thread d owns digit d: warp-exclusive prefixes and the tile count
    const int d = tid;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < SORT_THREADS / 32; ++w) {
        uint32_t c = s_whist[w][d];
        s_whist[w][d] = run;
        run += c;
    }
    const uint32_t tcount = run;
    const uint32_t tincl = block_scan_incl(tcount, s_warp);
    s_tstart[d] = tincl - tcount;
    const uint32_t gh = ghist[d];
    const uint32_t gincl = block_scan_incl(gh, s_warp);
    const uint32_t goff = gincl - gh;
    // publish the tile's count of digit d, then look back for the exclusive prefix
    uint32_t excl = 0;
    uint32_t* st = status + (size_t)tile * RADIX + d;
    if (tile == 0) {
        st_volatile(st, ST_PREFIX | tcount);
    } else {
        st_volatile(st, ST_AGG | tcount);
        excl = look_back(status + d, RADIX, tile, err);
        st_volatile(st, ST_PREFIX | ((excl + tcount) & ST_VALUE));
    }
    s_gbase[d] = goff + excl;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        if (dig[j] < RADIX) {
            uint32_t pos = s_tstart[dig[j]] + s_whist[warp][dig[j]] + rank[j];
            s_keys[pos] = key[j];
            s_vals[pos] = val[j];
        }
    }
    __syncthreads();
    const int tile_n = min(SORT_TILE, n - tile * SORT_TILE);
    for (int p = tid; p < tile_n; p += SORT_THREADS) {
        uint32_t k = s_keys[p];
        uint32_t dd = (k >> shift) & 255u;
        uint32_t o = s_gbase[dd] + (uint32_t)p - s_tstart[dd];
        if (o < (uint32_t)n) {  // always true unless a look-back gave up
            kout[o] = k;
            vout[o] = s_vals[p];
        }
    }
}

// keep the first (lowest triangle index) of every run of equal codes
__global__ void __launch_bounds__(SORT_THREADS)
k_unique(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int n, uint32_t* __restrict__ ucode,
         uint32_t* __restrict__ utri, uint32_t* status, uint32_t* counter, int n_tiles, BvhRoot* root,
         const uint32_t* __restrict__ mode, int* err) {
    if (skip_unique(*mode)) return;  // same codes: the last build's leaves stand
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_excl;
    __shared__ int s_tile;
    const int tid = threadIdx.x;
    if (tid == 0) s_tile = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int tile = s_tile;
    const int base = tile * SORT_TILE + tid * SORT_ITEMS;
    uint32_t fl = 0;
    uint32_t k[SORT_ITEMS];
    uint32_t prev = base > 0 && base - 1 < n ? keys[base - 1] : 0u;
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        int i = base + j;
        k[j] = i < n ? keys[i] : 0u;
        bool first = i < n && (i == 0 || k[j] != prev);
        fl |= (first ? 1u : 0u) << j;
        prev = k[j];
    }
    const uint32_t cnt = __popc(fl);
    const uint32_t incl = block_scan_incl(cnt, s_warp);
    if (tid == SORT_THREADS - 1) {
        uint32_t tsum = incl;
        uint32_t excl = 0;
        uint32_t* st = status + tile;
        if (tile == 0) {
            st_volatile(st, ST_PREFIX | tsum);
        } else {
            st_volatile(st, ST_AGG | tsum);
            excl = look_back(status, 1, tile, err);
            st_volatile(st, ST_PREFIX | ((excl + tsum) & ST_VALUE));
        }
        s_excl = excl;
        if (tile == n_tiles - 1) {
            root->n_leaves = (int)min(excl + tsum, (uint32_t)n);
            root->perm_valid = 1;  // k_build withdraws it if a wait of this LBVH build gave up
        }
    }
    __syncthreads();
    uint32_t o = s_excl + incl - cnt;
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        if (fl & (1u << j)) {
            if (o < (uint32_t)n) {  // always true unless a look-back gave up
                ucode[o] = k[j];
                utri[o] = vals[base + j];
            }
            ++o;
        }
    }
}

__device__ __forceinline__ int delta_at(const uint32_t* c, int i, int j, int n) {
    return (j < 0 || j >= n) ? -1 : __clz((int)(c[i] ^ c[j]));
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

constexpr int BUILD_LEAVES = 512;  // leaves per chunk (one CTA, one leaf per thread)

// Device view of the chunk summaries (see BvhBuffers).
struct ChunkView {
    int* cmin;
    float4* cbox;
    int2* srec;
    float4* sbox;
    int2* prec;
    float4* pbox;
    int* rcnt;
    int2* top;
    uint32_t* done;
    int lev_off[4];
};
constexpr int NLEV = 4;
constexpr int BIG_DELTA = 64;  // above every delta: a boundary that does not exist

// entries of each level for n leaves
__device__ __forceinline__ void level_counts(int n, int cnt[NLEV]) {
    cnt[0] = (n + BUILD_LEAVES - 1) / BUILD_LEAVES;
#pragma unroll
    for (int v = 1; v < NLEV; ++v) cnt[v] = (cnt[v - 1] + 31) / 32;
}

// Bottom-up build of the chunk-local nodes, and the chunk summaries.  Each CTA owns
// the BUILD_LEAVES sorted leaves [c0, c1) and stages delta of the boundaries
// c0 - 1 .. c1 - 1.  Phase 1 climbs through the nodes split inside the chunk
// (c0 <= g <= c1 - 2) in shared memory only: each child leaves its box, link and far
// range end in its side of the node's slot; the first to arrive stops, the second
// merges (A then B) and climbs on.  After the barrier the nodes both of whose
// children arrived are written out; a climb that stopped at a node whose other child
// lies in another chunk, or at a node split outside the chunk, writes its side into
// that node.  The remaining nodes span chunks; k_build_top finishes them from the
// chunk summaries written here:
//   * the boundaries that can end such a node's range inside this chunk: the strict
//     suffix minima of delta (the nearest smaller delta to the left of a node
//     further right) and the strict prefix minima (to the right of a node further
//     left), at most 30 each, with the union of the chunk's leaf boxes beyond /
//     up to each of them;
//   * the chunk's min delta and leaf box union (and, from the last CTA to finish,
//     the same per 32, 1024 and 32768 chunks);
//   * the nodes of the chunk that span chunks (no smaller delta on one side inside
//     the chunk, and the boundary to the next chunk).
__global__ void __launch_bounds__(BUILD_LEAVES)
k_build(const uint32_t* __restrict__ ucode, const uint32_t* __restrict__ utri, const float4* __restrict__ tri_box,
        const float4* __restrict__ tri_leaf, Node* nodes, float4* __restrict__ leaves, int2* range, BvhRoot* root,
        ChunkView cv, int* err) {
    __shared__ uint32_t s_flag[BUILD_LEAVES];  // bit 0: child A arrived, bit 1: child B
    // per node and side (A, B): lo (w = link), hi (w = far range end)
    __shared__ float4 s_lo[BUILD_LEAVES][2], s_hi[BUILD_LEAVES][2];
    __shared__ int s_delta[BUILD_LEAVES + 1];  // delta of boundary j at j - c0 + 1
    constexpr int W = BUILD_LEAVES / 32;
    __shared__ int s_wmin[W], s_wsr[W], s_wpr[W], s_wtop[W];  // per warp
    __shared__ float4 s_wlo[W], s_whi[W];
    // per warp, over the warps before (x*p) / after (x*s) it
    __shared__ int s_xpm[W], s_xsm[W], s_xos[W], s_xop[W], s_xot[W];
    __shared__ float4 s_xplo[W], s_xphi[W], s_xslo[W], s_xshi[W];
    __shared__ int s_nrec[3];
    __shared__ int s_last;
    const int tid = (int)threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nt = root->n_tris;
    const int n = min(root->n_leaves, nt);
    const int c0 = blockIdx.x * BUILD_LEAVES;
    const int c1 = min(c0 + BUILD_LEAVES, n);
    const int chunk = (int)blockIdx.x;
    if (blockIdx.x == 0 && tid == 0 && (*err & ERR_TIMEOUT)) root->perm_valid = 0;
    s_flag[tid] = 0u;
    const int i = c0 + tid;
    int l = i, r = i, link = ~i;  // the current subtree: leaf range, link
    float4 lo = ident_lo(), hi = ident_hi();
    bool live = i < n;  // still climbing
    int pend = -1;      // node where phase 1 stopped as the first local arrival
    int out = -1;       // node split outside the chunk where phase 1 stopped
    int dl = -1, dr = -1;
    bool is_a = false;
    uint32_t t = 0;  // the leaf's triangle (its box loads overlap the code loads below)
    if (live) {
        t = min(utri[i], (uint32_t)(nt - 1));
        lo = tri_box[2 * t];
        hi = tri_box[2 * t + 1];
    }
    {
        const int j = c0 + tid;
        s_delta[tid + 1] = delta_at(ucode, j, j + 1, n);  // -1 beyond the last leaf
        if (tid == 0) s_delta[0] = c0 < n ? delta_at(ucode, c0, c0 - 1, n) : -1;
    }
    __syncthreads();
    if (live && n == 1) {
        root->root = -1;
        root->top_lo = lo;
        root->top_hi = hi;
        live = false;
    }
    const float4 leaf_lo = lo, leaf_hi = hi;  // identity box for threads past the last leaf
    int level = 0;
    while (live) {
        if (++level > 64) {  // a climb is at most 31 levels over distinct 30-bit codes
            atomicOr(err, ERR_TIMEOUT);
            break;
        }
        dl = s_delta[l - c0];      // boundary l - 1
        dr = s_delta[r - c0 + 1];  // boundary r
        is_a = dr > dl;            // the parent extends to the right: this node is child A
        const int g = is_a ? r : l - 1;
        if (g < c0 || g > c1 - 2) {  // split outside the chunk
            out = g;
            break;
        }
        const int k = g - c0, side = is_a ? 0 : 1;
        s_lo[k][side] = make_float4(lo.x, lo.y, lo.z, __int_as_float(link));
        s_hi[k][side] = make_float4(hi.x, hi.y, hi.z, __int_as_float(is_a ? l : r));
        __threadfence_block();
        if (atomicOr(&s_flag[k], 1u << side) == 0u) {  // first to arrive: the sibling may be in another chunk
            pend = g;
            break;
        }
        __threadfence_block();
        // second to arrive: the sibling's side of the slot is complete
        const float4 olo = s_lo[k][side ^ 1], ohi = s_hi[k][side ^ 1];
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
            root->root = g;
            root->top_lo = lo;
            root->top_hi = hi;
            break;
        }
    }
    __syncthreads();
    if (i < n) {  // after the climbs: no global store is pending at their fences
        leaves[2 * i] = tri_leaf[2 * t];
        leaves[2 * i + 1] = tri_leaf[2 * t + 1];
    }
    // nodes of the chunk whose children both arrived here
    {
        const int g = c0 + tid;
        if (g <= c1 - 2 && s_flag[tid] == 3u) {
            const float4 alo = s_lo[tid][0], ahi = s_hi[tid][0], blo = s_lo[tid][1], bhi = s_hi[tid][1];
            const int la = __float_as_int(ahi.w), rb = __float_as_int(bhi.w);
            nodes[g].a_lo = alo;
            nodes[g].a_hi = make_float4(ahi.x, ahi.y, ahi.z, __int_as_float(s_delta[la - c0]));
            nodes[g].b_lo = blo;
            nodes[g].b_hi = make_float4(bhi.x, bhi.y, bhi.z, __int_as_float(s_delta[rb - c0 + 1]));
            range[g] = make_int2(la, rb);
        }
    }
    // a climb that stopped at a node another chunk completes: its side, in the node
    {
        int g = out;
        if (g < 0 && pend >= 0 && s_flag[pend - c0] != 3u) g = pend;
        if (g >= 0) write_side(nodes, range, g, is_a, lo, hi, link, l, r, is_a ? dl : dr);
    }
    if (c0 < n) {
        // thread tid: boundary j = c0 + tid (delta dk, BIG_DELTA past the last boundary)
        // and leaf c0 + tid (its box, the identity box past the last leaf)
        const int j = c0 + tid;
        const int dk = j <= n - 2 ? s_delta[tid + 1] : BIG_DELTA;
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
            s_wmin[warp] = pm;
            s_wlo[warp] = plo;
            s_whi[warp] = phi;
        }
        __syncthreads();
        if (tid < W) {  // exclusive prefix / suffix over the warps, for warp tid
            int a = BIG_DELTA, b = BIG_DELTA;
            float4 al = ident_lo(), ah = ident_hi(), bl = ident_lo(), bh = ident_hi();
            for (int w = 0; w < W; ++w) {
                if (w < tid) {
                    a = min(a, s_wmin[w]);
                    box_union(al, ah, s_wlo[w], s_whi[w]);
                } else if (w > tid) {
                    b = min(b, s_wmin[w]);
                    box_union(bl, bh, s_wlo[w], s_whi[w]);
                }
            }
            s_xpm[tid] = a;
            s_xsm[tid] = b;
            s_xplo[tid] = al;
            s_xphi[tid] = ah;
            s_xslo[tid] = bl;
            s_xshi[tid] = bh;
        }
        __syncthreads();
        const int wpm = s_xpm[warp], wsm = s_xsm[warp];
        // strict prefix (suffix) minimum: delta below every delta to its left (right)
        // in the chunk
        const int ppm = __shfl_up_sync(0xffffffffu, pm, 1), nsm = __shfl_down_sync(0xffffffffu, sm, 1);
        const int epm = min(wpm, lane > 0 ? ppm : BIG_DELTA);
        const int esm = min(wsm, lane < 31 ? nsm : BIG_DELTA);
        const bool pre = dk < epm, suf = dk < esm;
        // the chunk's leaves up to leaf j, and after it
        float4 up_lo = s_xplo[warp], up_hi = s_xphi[warp];
        box_union(up_lo, up_hi, plo, phi);
        float4 af_lo = s_xslo[warp], af_hi = s_xshi[warp];
        {
            const float4 nl = shfl_f4(slo, 1, false), nh = shfl_f4(shi, 1, false);
            if (lane < 31) box_union(af_lo, af_hi, nl, nh);
        }
        // node of boundary j spans chunks: no smaller delta on one side inside the chunk,
        // or j is the boundary to the next chunk
        const bool span = j <= n - 2 && (j == c1 - 1 || (s_flag[tid] != 3u));
        const unsigned bs = __ballot_sync(0xffffffffu, suf), bp = __ballot_sync(0xffffffffu, pre);
        const unsigned bt = __ballot_sync(0xffffffffu, span);
        if (lane == 0) {
            s_wsr[warp] = __popc(bs);
            s_wpr[warp] = __popc(bp);
            s_wtop[warp] = __popc(bt);
        }
        __syncthreads();
        if (tid < W) {
            int xs = 0, xp = 0, xt = 0, ts = 0, tp = 0, tt = 0;
            for (int w = 0; w < W; ++w) {
                if (w > tid) xs += s_wsr[w];
                if (w < tid) {
                    xp += s_wpr[w];
                    xt += s_wtop[w];
                }
                ts += s_wsr[w];
                tp += s_wpr[w];
                tt += s_wtop[w];
            }
            s_xos[tid] = xs;
            s_xop[tid] = xp;
            s_xot[tid] = xt;
            if (tid == 0) {
                s_nrec[0] = ts;
                s_nrec[1] = tp;
                s_nrec[2] = tt;
            }
        }
        __syncthreads();
        const int os = __popc(bs & ~((2u << lane) - 1u)) + s_xos[warp];
        const int op = __popc(bp & ((1u << lane) - 1u)) + s_xop[warp];
        const int ot = __popc(bt & ((1u << lane) - 1u)) + s_xot[warp];
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
            cv.rcnt[3 * chunk] = min(s_nrec[0], 32);
            cv.rcnt[3 * chunk + 1] = min(s_nrec[1], 32);
            cv.rcnt[3 * chunk + 2] = min(s_nrec[2], 64);
            cv.cmin[chunk] = min(wpm, pm);
            cv.cbox[2 * chunk] = up_lo;
            cv.cbox[2 * chunk + 1] = up_hi;
        }
        if (span && ot < 64) cv.top[64 * chunk + ot] = make_int2(j, dk);  // at most 61 per chunk
    }
    // the last CTA to finish sums the chunks up per 32, 1024 and 32768 chunks
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(cv.done, 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    int cnt[NLEV];
    level_counts(n, cnt);
    for (int v = 1; v < NLEV; ++v) {
        const int* mi = cv.cmin + cv.lev_off[v - 1];
        const float4* bi = cv.cbox + 2 * cv.lev_off[v - 1];
        for (int e = warp; e < cnt[v]; e += W) {
            const int k = 32 * e + lane;
            int m = BIG_DELTA;
            float4 blo = ident_lo(), bhi = ident_hi();
            if (k < cnt[v - 1]) {
                m = __ldcg(mi + k);
                blo = __ldcg(bi + 2 * k);
                bhi = __ldcg(bi + 2 * k + 1);
            }
            warp_box_reduce(blo, bhi);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) {
                cv.cmin[cv.lev_off[v] + e] = m;
                cv.cbox[2 * (cv.lev_off[v] + e)] = blo;
                cv.cbox[2 * (cv.lev_off[v] + e) + 1] = bhi;
            }
        }
        __syncthreads();
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
        const bool hit = (right ? e > idx : e < idx) && e < cnt[v] && __ldg(m + e) < d;
        unsigned b = __ballot_sync(0xffffffffu, hit);
        if (b) {
            int f = right ? base + __ffs(b) - 1 : base + 31 - __clz(b);
            for (int u = v - 1; u >= 0; --u) {  // descend: the first qualifying entry of group f
                const int b2 = 32 * f, e2 = b2 + lane;
                const bool h2 = e2 < cnt[u] && __ldg(cv.cmin + cv.lev_off[u] + e2) < d;
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
    const int2 q = lane < count ? __ldg(rec + lane) : make_int2(0, BIG_DELTA);
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
            for (int e = a + lane; e <= b; e += 32) box_union(ul, uh, __ldg(bx + 2 * e), __ldg(bx + 2 * e + 1));
            break;
        }
        const int e1 = a + lane, e2 = (b & ~31) + lane;
        if (e1 <= (a | 31)) box_union(ul, uh, __ldg(bx + 2 * e1), __ldg(bx + 2 * e1 + 1));
        if (e2 <= b) box_union(ul, uh, __ldg(bx + 2 * e2), __ldg(bx + 2 * e2 + 1));
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
// enters its parent (the range end with the larger delta) as build_internal's climb
// would have put it there.
constexpr int TOP_WARPS = 8;
__global__ void __launch_bounds__(TOP_WARPS * 32)
k_build_top(ChunkView cv, Node* nodes, int2* range, BvhRoot* root, int* err) {
    const int nt = root->n_tris;
    const int n = min(root->n_leaves, nt);
    int cnt[NLEV];
    level_counts(n, cnt);
    const int lane = (int)(threadIdx.x & 31u);
    // each chunk's nodes that span chunks sit in its 64 slots; iteration `it` takes slot
    // it / F of chunk it % F, so the (few, low) occupied slots spread over all warps
    const uint32_t F = (uint32_t)cnt[0], slots = 64u * F;
    const uint32_t nw = gridDim.x * TOP_WARPS;
    for (uint32_t it = blockIdx.x * TOP_WARPS + (threadIdx.x >> 5); it < slots; it += nw) {
        const uint32_t ch = it % F, sl = it / F;
        if ((int)sl >= __ldg(cv.rcnt + 3 * ch + 2)) continue;
        const int2 item = __ldg(cv.top + 64 * ch + sl);
        const int g = item.x, d = item.y, c = g / BUILD_LEAVES;
        if (g < 0 || g > n - 2 || c >= cnt[0]) {
            if (lane == 0) atomicOr(err, ERR_TIMEOUT);
            continue;
        }
        // left end: boundary jl (leaves from jl + 1), -1 = none
        int2 q;
        int jl = -1, dlft = -1, cl = -1;
        float4 lo = ident_lo(), hi = ident_hi();
        int k = first_record(cv.srec + 32 * c, __ldg(cv.rcnt + 3 * c), g, d, false, lane, q);
        int cc = c;
        if (k < 0) {
            cc = nearest_chunk(cv, cnt, c, d, false, lane, err);
            if (cc >= 0) k = first_record(cv.srec + 32 * cc, __ldg(cv.rcnt + 3 * cc), -1, d, false, lane, q);
        }
        if (k >= 0) {
            jl = q.x;
            dlft = q.y;
            cl = cc;
            box_union(lo, hi, __ldg(cv.sbox + 2 * (32 * cc + k)), __ldg(cv.sbox + 2 * (32 * cc + k) + 1));
        }
        // right end: boundary jr (leaves up to jr), n - 1 = none
        int jr = n - 1, drgt = -1, cr = cnt[0] - 1;
        k = first_record(cv.prec + 32 * c, __ldg(cv.rcnt + 3 * c + 1), g, d, true, lane, q);
        cc = c;
        if (k < 0) {
            cc = nearest_chunk(cv, cnt, c, d, true, lane, err);
            if (cc >= 0) k = first_record(cv.prec + 32 * cc, __ldg(cv.rcnt + 3 * cc + 1), -1, d, true, lane, q);
        }
        if (k >= 0) {
            jr = q.x;
            drgt = q.y;
            cr = cc;
            box_union(lo, hi, __ldg(cv.pbox + 2 * (32 * cc + k)), __ldg(cv.pbox + 2 * (32 * cc + k) + 1));
        } else {
            box_union(lo, hi, __ldg(cv.cbox + 2 * cr), __ldg(cv.cbox + 2 * cr + 1));  // the last chunk
        }
        chunk_union(cv, cnt, cl + 1, cr - 1, lane, lo, hi);
        if (lane == 0) {
            if (jl < 0 && jr == n - 1) {
                root->root = g;
                root->top_lo = lo;
                root->top_hi = hi;
            } else {
                const bool is_a = drgt > dlft;
                write_side(nodes, range, is_a ? jr : jl, is_a, lo, hi, g, jl + 1, jr, is_a ? dlft : drgt);
            }
        }
    }
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

}  // namespace

void BvhBuffers::plan(Arena& a, int nv_, int nt_, bool normals) {
    nv = nv_;
    nt = nt_;
    has_normals = normals;
    tiles_sort = nt > 0 ? cdiv(nt, SORT_TILE) : 0;
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
    // histograms | sort status (PASSES x tiles x RADIX) | sort counters | unique status | unique counter
    // | rebuild mode word | finished chunk CTAs
    scratch_words = (size_t)PASSES * RADIX + (size_t)PASSES * tiles_sort * RADIX + PASSES + tiles_sort + 3;
    a.want(&scratch, scratch_words);
}

namespace {
// Self-test of the look-back's bounded wait: one thread looks back from tile 1 at a
// status word (tile 0's) that nothing publishes; the walk gives up after SPIN_LIMIT
// sleeps, records ERR_TIMEOUT and returns.
__global__ void k_selftest_look_back(const uint32_t* status, int* err) {
    if (threadIdx.x == 0) (void)look_back(status, 1, 1, err);
}
}  // namespace

cudaError_t launch_selftest_look_back(const uint32_t* zero_status, int* err, cudaStream_t s) {
    k_selftest_look_back<<<1, 32, 0, s>>>(zero_status, err);
    return cudaGetLastError();
}

cudaError_t lbvh_build(BvhBuffers& b, float thickness, float box_depth, int* d_err, cudaStream_t s) {
    if (b.nt == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(b.scratch, 0, b.scratch_words * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    uint32_t* ghist = b.scratch;
    uint32_t* sstat = ghist + PASSES * RADIX;
    uint32_t* scount = sstat + (size_t)PASSES * b.tiles_sort * RADIX;
    uint32_t* ustat = scount + PASSES;
    uint32_t* ucount = ustat + b.tiles_sort;
    uint32_t* mode = ucount + 1;
    ChunkView cv{b.cmin, b.cbox, b.srec, b.sbox, b.prec, b.pbox, b.rcnt, b.top, mode + 1,
                 {b.lev_off[0], b.lev_off[1], b.lev_off[2], b.lev_off[3]}};
    k_body_prep<<<cdiv(b.nv, BUILD_THREADS), BUILD_THREADS, 0, s>>>(b.xyz_in, b.has_normals ? b.nrm_in : nullptr,
                                                                     b.nv, thickness, b.verts, b.root, b.nt);
    k_tri_boxes<<<cdiv(b.nt, BUILD_THREADS), BUILD_THREADS, 0, s>>>(b.verts, b.nv, b.tris, b.nt, box_depth, b.tri_box,
                                                                     b.tri_leaf, b.root, d_err);
    k_morton<<<cdiv(b.nt, BUILD_THREADS), BUILD_THREADS, 0, s>>>(b.tri_box, b.nt, b.root, b.codes, ghist);
    if (b.coherent)
        k_coherence<<<cdiv(b.nt, BUILD_THREADS), BUILD_THREADS, 0, s>>>(b.codes, b.keys[1], b.vals[1], b.nt, b.root,
                                                                         mode);
    const uint32_t* kin = b.codes;
    const uint32_t* vin = nullptr;
    for (int p = 0; p < PASSES; ++p) {
        uint32_t* ko = b.keys[p & 1];
        uint32_t* vo = b.vals[p & 1];
        k_sort_pass<<<b.tiles_sort, SORT_THREADS, 0, s>>>(kin, vin, ko, vo, b.nt, 8 * p, ghist + p * RADIX,
                                                          sstat + (size_t)p * b.tiles_sort * RADIX, scount + p, mode, d_err);
        kin = ko;
        vin = vo;
    }
    k_unique<<<b.tiles_sort, SORT_THREADS, 0, s>>>(kin, vin, b.nt, b.ucode, b.utri, ustat, ucount, b.tiles_sort,
                                                   b.root, mode, d_err);
    k_build<<<b.chunks, BUILD_LEAVES, 0, s>>>(b.ucode, b.utri, b.tri_box, b.tri_leaf, b.nodes, b.leaves, b.range,
                                               b.root, cv, d_err);
    if (b.chunks > 1)  // else the whole tree is one chunk's
        k_build_top<<<std::min(cdiv(64 * b.chunks, TOP_WARPS), 1024), TOP_WARPS * 32, 0, s>>>(cv, b.nodes, b.range,
                                                                                              b.root, d_err);
    return cudaGetLastError();
}

}  // namespace visg
