// visg_internal.cuh — device data layout and host-side engine of the cloth step.
//
// HBM layout (all arrays 16-byte aligned, one allocation per engine):
//   cloth state, double-buffered: 2 float4 per vertex
//        [x.x x.y x.z v.x] [v.y v.z flags margin]        32 B, one sector per gather
//        v = (x - x_old) / dt, computed once per step by the vertex's own thread;
//        with StepParams::drec the record carries D = x - x_old in its place (then
//        no spring reads a neighbour's velocity and the step needs only x - x_old);
//        x_old is x (flag XO_IS_X) or the x of the same vertex in the other buffer;
//        the last word is the query cache's margin: while the vertex stays within
//        that distance of where its last first-hit query was answered, the answer
//        (no leaf, or with flag LEAF_CACHED the leaf in the flags word's bits 3-31)
//        still holds (0 = none); the leaf travels in the record, so a vertex whose
//        answer is cached reads no other per-vertex array to find it
//   contact normal (previous step):  float4 per vertex, read only when flags says so
//   rowp:   u32 per vertex + 1, merged CSR row offsets; bit 31 = vertex pinned
//   ent:    uint2 per directed spring {end | list << 30, rest}         8 B
//   kent:   f32 per directed spring, only with per-spring stiffness
//   sell:   the same springs in sliced-ELL order for the step kernel: a slice is 32
//           consecutive vertices of one garment, padded to its longest row; entry k of
//           lane l of slice s sits at slice_off[s] + 32 k + l, so the k-th springs of a
//           warp are one contiguous 256-byte run (sellk: stiffness, same layout)
//   vcount: uint2 per vertex: the row's springs per list (16 bits each, list 3 15
//           bits), bit 31 of .y = pinned
//   tiles:  int4 per tile {garment, first vertex, end vertex, first slice}; a tile
//           never straddles two garments.  twin: int2 per tile {first entry, count},
//           the tile's contiguous sliced-ELL block, which a TMA bulk copy stages in
//           shared memory; count 0 = read from global memory
//   per body: LBVH nodes (64 B: both children's boxes and links), leaves (32 B:
//           v0 and the face normal), root record; build scratch (sort buffers,
//           look-back status words, chunk summaries)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/visg_sim.h"
#include "visg_math.cuh"

namespace visg {

void set_last_error(const char* msg);  // what visg_last_error returns next

constexpr uint32_t PIN_BIT = 0x80000000u;
constexpr uint32_t ROW_MASK = 0x7fffffffu;
constexpr uint32_t END_MASK = 0x3fffffffu;
constexpr int LIST_SHIFT = 30;
constexpr uint32_t FLAG_HAS_NORMAL = 1u;  // the previous contact normal is stored (non-zero)
constexpr uint32_t FLAG_XO_IS_X = 2u;     // x_old equals x (else x_old = x of the other buffer)
constexpr uint32_t FLAG_LEAF_CACHED = 4u; // the query cache's answer is the leaf in bits 3-31 (else no leaf)
constexpr int LEAF_SHIFT = 3;                // the cached leaf's position in the flags word
constexpr int kLeafCacheMax = 1 << 29;       // leaves from this index on are not cached (they do not fit)

// tile descriptor .x: the garment, and whether it has a body (set at finalize: a body
// has at least one triangle, so every build of its tree has leaves)
constexpr int TILE_GARMENT = 0x3fffffff;
constexpr int TILE_BODY = 0x40000000;

// error bits written by kernels into the engine's error word
constexpr int ERR_STACK = 1;     // traversal stack would overflow (not reachable for <= 30-bit codes)
constexpr int ERR_DIVERGED = 2;  // divergence check tripped
constexpr int ERR_TIMEOUT = 4;   // a bounded look-back wait gave up
constexpr int ERR_INDEX = 8;     // an index read on the device was out of range (not used as one)

// LBVH internal node: children's boxes and links.  Links: >= 0 internal node,
// < 0 leaf ~link.  Each child writes its own two float4 during the build.
struct __align__(16) Node {
    float4 a_lo;  // child A min xyz, w = link A
    float4 a_hi;  // child A max xyz
    float4 b_lo;  // child B min xyz, w = link B
    float4 b_hi;  // child B max xyz
};

struct __align__(16) BvhRoot {
    int root;      // root internal node, -1 when there are fewer than two leaves
    int n_leaves;  // T' (after de-duplication)
    int n_tris;    // T
    int perm_valid;  // codes and keys/vals[sorted] hold the last build's codes and sorted list
    float4 frame_lo, frame_hi;  // Morton frame: identity box U every expanded triangle box
    float4 top_lo, top_hi;      // box of the root node (identity U children), or of the only leaf
    int sorted;                 // which of the two sort buffers holds the last build's list
    int pad_[3];
};

// device view of one body's LBVH, as the step and query kernels use it
struct BvhView {
    const Node* nodes;
    const float4* leaves;  // 2 per leaf: (v0.xyz, n.x) (n.y, n.z, triangle, 0)
    const BvhRoot* root;
};

// ---- host: simple bump allocator over one cudaMalloc --------------------------------
struct Arena {
    char* base = nullptr;
    size_t size = 0, used = 0;
    std::vector<std::pair<void**, size_t>> plan;
    template <typename T>
    void want(T** p, size_t count) { plan.push_back({(void**)p, ((count * sizeof(T) + 255) / 256) * 256}); }
    cudaError_t commit();
    void release();
};

// ---- LBVH buffers of one body ----------------------------------------------------------
struct BvhBuffers {
    int nv = 0, nt = 0;        // body vertices, triangles
    int tiles_sort = 0;        // look-back tiles of one radix pass
    bool has_normals = false;
    bool coherent = false;     // merge the changed codes into the last build's sorted list
    float* xyz_in = nullptr;   // nv*3 staging (upload target)
    float* nrm_in = nullptr;   // nv*3 staging
    float4* verts = nullptr;   // nv, thickness push applied
    uint32_t* tris = nullptr;  // nt*3
    float4* tri_box = nullptr;   // 2*nt (min, max)
    float4* tri_leaf = nullptr;  // 2*nt (v0, n)
    uint32_t* codes = nullptr;   // nt, per triangle
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* vals[2] = {nullptr, nullptr};
    uint32_t* ucode = nullptr;   // T'
    uint32_t* utri = nullptr;    // T'
    Node* nodes = nullptr;       // nt-1
    float4* leaves = nullptr;    // 2*nt
    int2* range = nullptr;       // nt-1 leaf range of each internal node
    // Summaries of the 512-leaf chunks for the nodes whose leaf range spans chunks
    // (levels: per chunk, per 32 chunks, per 1024, per 32768, at lev_off[0..3])
    int* cmin = nullptr;         // min delta over the boundaries of the entry's chunks
    float4* cbox = nullptr;      // 2 per entry: union of the entry's leaf boxes
    int2* srec = nullptr;        // 32 per chunk: suffix-minimum boundaries {position, delta}, right to left
    float4* sbox = nullptr;      // 2 per record: union of the chunk's leaves after the boundary
    int2* prec = nullptr;        // 32 per chunk: prefix-minimum boundaries, left to right
    float4* pbox = nullptr;      // 2 per record: union of the chunk's leaves up to the boundary
    int* rcnt = nullptr;         // 3 per chunk: suffix and prefix record counts, nodes in `top`
    int2* top = nullptr;         // 64 per chunk: {boundary, delta} of the nodes that span chunks
    int chunks = 0;              // chunks of nt leaves
    int lev_off[4] = {0, 0, 0, 0};
    BvhRoot* root = nullptr;
    uint32_t* scratch = nullptr; // radix histograms, look-back status words, tile counters (the build clears them)
    size_t scratch_words = 0;
    int max_ctas = 0;            // CTAs a build launches at most (one per 512 triangles)
    float* part = nullptr;       // 8 per CTA: the CTA's box union
    uint32_t* ucnt = nullptr;    // per CTA: distinct codes in its slice
    uint32_t* chg = nullptr;     // count + the triangles whose code changed since the last build
    uint32_t* sync = nullptr;    // grid-barrier counters, zero between builds
    uint32_t* gdone = nullptr;   // per summary entry above level 0: members finished
    int n_entries = 0;           // summary entries of all levels

    void plan(Arena& a, int nv_, int nt_, bool normals);
    BvhView view() const { return BvhView{nodes, leaves, root}; }
};

// The full device build in one cooperative launch: vertex push -> boxes + frame ->
// Morton codes -> sort (merge of the changed codes, or 4 radix passes) ->
// de-duplication -> bottom-up build + refit.  The body's vertices (and normals) are
// read from xyz / nrm when given (device memory, read in stream order), else from
// the staging buffers; with margin_state, the same launch voids the query-cache
// margins of cloth vertices [m0, m1).
cudaError_t lbvh_build(BvhBuffers& b, float thickness, float box_depth, int* d_err, cudaStream_t s,
                       const float* xyz = nullptr, const float* nrm = nullptr, float4* margin_state = nullptr,
                       int64_t m0 = 0, int64_t m1 = 0);

// ---- step kernel arguments ---------------------------------------------------------------
struct StepParams {
    float dt, mass, gx, gy, gz, damp, kd, gamma;
    float list_k[VISG_MAX_LISTS];
    int n_lists;
    float max_disp;
    int margin;  // keep each vertex's proven distance to its body's leaf boxes (collision margin)
    int drec;    // records carry D = x - x_old instead of v (spring damping +0, Verlet damping != 1)
    float dmax;  // tame bound on |D| (|v| = |D| / dt < 1e15)
};

struct StepArgs {
    const float4* state_in;
    float4* state_out;
    float4* normal;  // in place
    const uint32_t* rowp;
    const uint2* ent;
    const float* kent;
    const int4* tiles;
    int n_tiles;
    const BvhView* bodies;  // per garment
    int* err;
    uint32_t* check;  // [0] max |dx| bits, [1] non-finite count
    int2* cand;       // split collision: {vertex, garment} of the vertices inside their body's box
    uint32_t* cand_count;
    const uint2* sell;        // sliced-ELL springs (see the layout above)
    const float* sellk;       // per-entry stiffness in the same layout, with SV_PERK
    const uint32_t* slice_off;
    const uint2* vcount;      // per vertex: springs per list, 16 bits each (list 3: 15), bit 63 = pinned
    uint32_t* wild;           // sticky: some record had |x| or |v| >= 1e15 (or NaN)
    const int2* twin;         // per tile sliced-ELL block, with SV_STAGED
    int win_cap;              // entries per shared-memory stage buffer
    StepParams p;
};

enum StepVariant : int {
    SV_PERK = 1,      // per-spring stiffness array
    SV_REFV = 2,      // reference Verlet expression (gamma == 1)
    SV_COLLIDE = 4,   // body collision
    SV_CHECK = 8,     // divergence check
    SV_KD0 = 16,      // spring damping exactly +0
    SV_SPLIT = 32,    // collision in its own kernel over a compacted candidate list
    SV_STAGED = 64,   // sliced-ELL blocks staged in shared memory by TMA bulk copies
};
// dynamic shared memory of a launch: two stage buffers of win_cap entries + barriers
int step_smem_bytes(int variant, int win_cap);
cudaError_t launch_step(const StepArgs& a, int variant, int block, int grid, cudaStream_t s);
// record `before` / `after` around every step-kernel launch this thread issues (null: stop)
void set_step_timing(cudaEvent_t before, cudaEvent_t after);
int step_max_ctas_per_sm(int variant, int block, int win_cap);

// self-tests of the bounded waits: each must give up and set ERR_TIMEOUT in *err
cudaError_t launch_selftest_mbar_wait(int* err, cudaStream_t s);
cudaError_t launch_selftest_look_back(const uint32_t* zero_status, int* err, cudaStream_t s);
cudaError_t launch_selftest_grid_wait(uint32_t* zero_counter, int* err, cudaStream_t s);
// exhaustive check of the packed square root and reciprocal: cnt[3] = {checked, bad roots, bad reciprocals}
cudaError_t launch_selftest_exact_math(unsigned long long* cnt, cudaStream_t s);

// first-hit queries of external points against one body
cudaError_t launch_query(BvhView v, const float* pts, int n, int* leaf, int* inside, float* dist,
                         float* normal, int* err, cudaStream_t s);

// unpack positions of vertices [0, n) into packed xyz
cudaError_t launch_unpack_positions(const float4* state, int64_t n, float* out, cudaStream_t s);
cudaError_t launch_unpack_state(const float4* state, const float4* other, const float4* normal, int64_t n, float* x,
                                float* xo, float* nrm, cudaStream_t s);
// x/xo/nrm may be NULL (kept); dt recomputes v = (x - x_old) / dt
cudaError_t launch_pack_state(float4* state, float4* other, float4* normal, int64_t n, const float* x,
                              const float* xo, const float* nrm, float dt, int drec, float dmax, uint32_t* wild,
                              cudaStream_t s);

// output stage: pos4 = (x, 1) of st_now; fn = face normals of st_prev; vn = normalised
// sums of each vertex's face normals (row/col: vertex -> face CSR).  NULL skips one.
// colour (with rgb, the object colour): the SH-shaded colour of each vertex normal
cudaError_t launch_render(const float4* st_now, const float4* st_prev, int64_t n, const uint32_t* faces, int64_t nf,
                          const uint32_t* row, const uint32_t* col, float* fn, float4* pos4, float* vn, float* colour,
                          const float* rgb, cudaStream_t s);

// forget the collision margin of vertices [v0, v1) (their body moved)
cudaError_t launch_clear_margin(float4* state, int64_t v0, int64_t v1, cudaStream_t s);

// number of vertices with the contact flag set, accumulated into *count
cudaError_t launch_count_contacts(const float4* state, int64_t n, unsigned long long* count, cudaStream_t s);

// scatter (idx[k] -> x = x_old = xyz[k]) into the state, keeping the contact flag
cudaError_t launch_set_vertices(float4* state, const uint32_t* idx, const float* xyz, int n, float dt, uint32_t* wild,
                                cudaStream_t s);

// set *wild when some record of [0, n) has a component of |x| or |v| >= 1e15 (or NaN)
cudaError_t launch_check_tame(const float4* state, int64_t n, uint32_t* wild, cudaStream_t s);

// ---- adjoint ----------------------------------------------------------------------------
// Packed float3 arrays of one recorded step: x, x_old and the contact normal entering
// the step (n_in), and the contact normals the step produced (n_out: non-zero = the
// vertex was projected, with that plane normal).
struct AdjArgs {
    const double* x;
    const double* xo;
    const double* n_in;
    const double* n_out;
    const uint32_t* rowp;
    const uint2* ent;
    const float* kent;     // per entry stiffness, or NULL (list stiffness)
    const uint32_t* rev;   // reverse entry of every directed spring
    const double* lx_in;   // adjoint of the step's outputs x', x_old' (double3 per vertex)
    const double* lxo_in;
    double* lx_out;        // adjoint of the step's inputs x, x_old
    double* lxo_out;
    double* G;             // adjoint of the force on each vertex (double3)
    double* dk;            // per entry, accumulated over steps
    double* dscalar;       // [3]: gamma, force damping, spring damping; accumulated
    int n;
    StepParams p;
};
cudaError_t launch_adjoint_step(const AdjArgs& a, cudaStream_t s);
// the differentiable forward: one step in double (packed double3 arrays)
cudaError_t launch_step_f64(const double* x, const double* xo, double* xn, double* xon, double* nrm,
                            const uint32_t* rowp, const uint2* ent, const float* kent, const BvhView* bodies,
                            const float4* body_verts, const uint32_t* body_tris, const StepParams& p, int refv,
                            int collide, int n, int* err, unsigned* contacts, cudaStream_t s);
cudaError_t launch_widen(const float* src, double* dst, int64_t n, cudaStream_t s);
cudaError_t launch_narrow(const double* src, float* dst, int64_t n, cudaStream_t s);

}  // namespace visg
