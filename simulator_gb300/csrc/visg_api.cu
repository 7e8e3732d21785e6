// visg_api.cu — the C ABI of include/visg_sim.h over one engine type.
//
// An Engine holds G >= 1 garments, each with its own body: the plain form
// (VisgSim, the reference's Simulator, src/simulator.h:9-59) is an engine with one
// garment; the batched form (VisgBatch) is the same engine with many.  All device
// memory of an engine is one allocation carved by an Arena.  Steps are launched
// on the user's stream; multi-step loops are replayed from CUDA graphs captured on
// an internal stream (two graphs, one per ping-pong parity).
#include <cuda_runtime.h>

#include <cmath>

#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "visg_internal.cuh"

#include <nvtx3/nvToolsExt.h>  // header-only: the ranges cost nothing unless a profiler attaches

using namespace visg;

namespace {

thread_local std::string g_err = "";

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

}  // namespace

// the message visg_last_error returns, for the host-only translation units
void visg::set_last_error(const char* msg) { g_err = msg; }

namespace {

int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? VISG_ERR_OOM : VISG_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CU(call)                                          \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

constexpr int kNumBlocks = 4;
constexpr int kBlocks[kNumBlocks] = {128, 256, 512, 1024};
// largest sliced-ELL block (entries) a tile of each block size may stage in shared
// memory: 16 entries per vertex (14 for 1024, whose two buffers must fit the 227 KB a
// CTA may hold); two buffers take 32 / 64 / 128 / 224 KB
constexpr int kStageCap[kNumBlocks] = {2048, 4096, 8192, 14336};
int block_index(int b) {
    for (int i = 0; i < kNumBlocks; ++i)
        if (kBlocks[i] == b) return i;
    return -1;
}

struct GarmentIn {
    std::vector<float> xyz;
    int N = 0;
    std::vector<std::vector<uint32_t>> rows;
    std::vector<std::vector<VisgSpring>> ents;
    std::vector<std::vector<float>> ks;
    std::vector<uint32_t> pinned;
    std::vector<float> bxyz, bnrm;
    int nv = 0, nt = 0;
    std::vector<uint32_t> tris;
};

int validate_params(const VisgParams* p) {
    if (!p) return fail(VISG_ERR_INVALID_ARG, "params is NULL");
    if (p->n_lists < 1 || p->n_lists > VISG_MAX_LISTS) return fail(VISG_ERR_INVALID_ARG, "n_lists must be 1..4");
    if (!(p->dt > 0.0f) || !(p->mass > 0.0f)) return fail(VISG_ERR_INVALID_ARG, "dt and mass must be > 0");
    return VISG_OK;
}

}  // namespace

namespace visg {

cudaError_t Arena::commit() {
    size = 0;
    for (auto& pl : plan) size += pl.second;
    if (size == 0) size = 256;
    cudaError_t e = cudaMalloc((void**)&base, size);
    if (e != cudaSuccess) {
        base = nullptr;
        return e;
    }
    e = cudaMemset(base, 0, size);
    if (e != cudaSuccess) return e;
    used = 0;
    for (auto& pl : plan) {
        *pl.first = base + used;
        used += pl.second;
    }
    plan.clear();
    return cudaSuccess;
}

void Arena::release() {
    if (base) cudaFree(base);
    base = nullptr;
    size = used = 0;
}

}  // namespace visg

struct Engine {
    VisgParams p{};
    cudaStream_t stream = nullptr;
    cudaStream_t cap = nullptr;
    cudaStream_t cap2 = nullptr;  // the second group's capture stream
    cudaStream_t run2 = nullptr;  // the second group's stream outside graphs
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr, fork2 = nullptr, join2 = nullptr;
    // garment groups stepped as independent chains: group 1 starts at garment
    // boundary vsplit (vertex), i.e. at tile tsplit[b] of each tile table
    int tsplit[kNumBlocks] = {0, 0, 0, 0};
    int64_t vsplit = 0;
    bool finalized = false;
    std::vector<GarmentIn> gin;
    int G = 0;
    int64_t N = 0, E = 0;
    std::vector<int64_t> voff, eoff;
    std::vector<int64_t> merged_pos;  // merged entry -> index in (garment, list, entry) order
    std::vector<uint32_t> h_rowp;
    bool perk = false, any_body = false;
    Arena arena;
    float4* d_state[2] = {nullptr, nullptr};
    float4* d_normal = nullptr;
    uint32_t* d_rowp = nullptr;
    uint2* d_ent = nullptr;
    float* d_k = nullptr;
    int4* d_tiles[kNumBlocks] = {nullptr, nullptr, nullptr, nullptr};
    int n_tiles[kNumBlocks] = {0, 0, 0, 0};
    int2* d_twin[kNumBlocks] = {nullptr, nullptr, nullptr, nullptr};  // per tile sliced-ELL block {first entry, count}
    int win_cap[kNumBlocks] = {0, 0, 0, 0};                           // entries per stage buffer, 0 = no tile staged
    uint2* d_sell = nullptr;                         // sliced-ELL springs
    float* d_sellk = nullptr;
    uint32_t* d_slice_off = nullptr;
    uint2* d_vcount = nullptr;                      // springs per list | pin bit, per vertex
    std::vector<uint2> h_vcount;
    uint32_t* d_wild = nullptr;                      // sticky: a record was not tame
    int stage = 0;                                   // stage sliced-ELL blocks (autotuned)
    BvhView* d_views = nullptr;
    std::vector<BvhBuffers> bvh;
    int* d_err = nullptr;
    uint32_t* d_check = nullptr;
    int2* d_cand = nullptr;            // split collision: queued candidates
    uint32_t* d_cand_count = nullptr;
    // output stage: faces of each garment (local indices), and on the device all
    // garments' faces with global indices, the vertex -> face CSR, the face normals
    std::vector<std::vector<uint32_t>> gfaces;
    uint32_t* d_faces = nullptr;
    uint32_t* d_frow = nullptr;
    uint32_t* d_fcol = nullptr;
    float* d_fnorm = nullptr;
    int64_t NF = 0;
    bool prev_ok = false;  // the other buffer holds the positions the last step started from
    int split = 1;                     // collision in its own kernel (autotuned)
    float* d_stage = nullptr;  // 10*N floats
    uint32_t* h_status = nullptr;  // pinned: err, check0, check1
    int cur = 0;
    int block = 256, grid = 0;
    // SMs the persistent step kernel leaves free when two garment groups step as
    // overlapping chains: one group's collision pass then runs beside the other
    // group's step kernel instead of after it (chosen by the autotuner)
    int reserve = 0;
    int64_t steps_since_check = 0;
    cudaGraphExec_t chunk_exec[2] = {nullptr, nullptr};
    int chunk_steps = 16;
    int sm_count = 0;
    // adjoint records
    struct Adj {
        int ckpt = 0, nsteps = 0;
        std::vector<double*> ck;     // FP64 checkpoints: x, x_old, normal (9N doubles) every ckpt steps
        double* s64 = nullptr;       // FP64 state: [x0 | xo0 | x1 | xo1 | n] (15N doubles)
        double* rec = nullptr;       // (ckpt + 1) recorded states of the segment being replayed
        double* lam = nullptr;       // 4 x 3N: adjoints of x, x_old (in / out)
        double* G = nullptr;         // 3N
        double* dk = nullptr;        // per merged entry
        double* dsc = nullptr;       // 3
        uint32_t* rev = nullptr;     // reverse entry of every merged entry
        unsigned* contacts = nullptr;  // vertices projected in each forward step
        bool ready = false;
    } adj;

    // asynchronous position read-back: two device staging slots copied to host memory
    // on their own stream while later steps run
    static constexpr int kReadSlots = 3;  // reads in flight at most
    struct Readback {
        cudaStream_t copy = nullptr;
        float* d_pos[kReadSlots] = {};
        cudaEvent_t unpacked[kReadSlots] = {}, copied[kReadSlots] = {};
        uint32_t* h_err = nullptr;  // pinned: the error word as of each slot's read
        bool used[kReadSlots] = {};
        int next = 0;     // slot of the next read
        int pending = 0;  // reads issued and not yet waited for (0..kReadSlots)
    } rb;

    ~Engine() {
        if (stream) cudaStreamSynchronize(stream);
        cudaDeviceSynchronize();
        for (int k = 0; k < kReadSlots; ++k) {
            if (rb.d_pos[k]) cudaFree(rb.d_pos[k]);
            if (rb.unpacked[k]) cudaEventDestroy(rb.unpacked[k]);
            if (rb.copied[k]) cudaEventDestroy(rb.copied[k]);
        }
        if (rb.copy) cudaStreamDestroy(rb.copy);
        free_faces();
        if (rb.h_err) cudaFreeHost(rb.h_err);
        destroy_graphs();
        if (d_sv_idx) cudaFree(d_sv_idx);
        if (h_sv) cudaFreeHost(h_sv);
        if (sv_done) cudaEventDestroy(sv_done);
        free_adjoint();
        arena.release();
        if (h_status) cudaFreeHost(h_status);
        if (cap) cudaStreamDestroy(cap);
        if (cap2) cudaStreamDestroy(cap2);
        if (run2) cudaStreamDestroy(run2);
        for (cudaEvent_t ev : {fork_ev, join_ev, fork2, join2})
            if (ev) cudaEventDestroy(ev);
    }

    void destroy_graphs() {
        for (int c = 0; c < 2; ++c)
            if (chunk_exec[c]) {
                cudaGraphExecDestroy(chunk_exec[c]);
                chunk_exec[c] = nullptr;
            }
    }

    void free_adjoint() {
        for (auto* q : adj.ck) cudaFree(q);
        adj.ck.clear();
        void* ps[] = {adj.s64, adj.rec, adj.lam, adj.G, adj.dk, adj.dsc, adj.rev, adj.contacts};
        for (void* q : ps)
            if (q) cudaFree(q);
        adj = Adj();
    }

    int add(const float* cloth, int n, const uint32_t* const* rows, const VisgSpring* const* csr,
            const float* const* list_k, const uint32_t* pinned, int n_pinned, const float* body, const float* bn,
            int nv, const uint32_t* tris, int nt, int* gid) {
        if (finalized) return fail(VISG_ERR_STATE, "garments can only be added before finalize");
        if (!cloth || n <= 0) return fail(VISG_ERR_INVALID_ARG, "cloth_xyz is NULL or n_vertices <= 0");
        if (!rows || !csr) return fail(VISG_ERR_INVALID_ARG, "csr_row/csr is NULL");
        if (nt < 0 || nv < 0 || (nt > 0 && (!body || !tris || nv <= 0)))
            return fail(VISG_ERR_INVALID_ARG, "body arrays are NULL or sizes negative");
        if (N + n > (int64_t)END_MASK) return fail(VISG_ERR_INVALID_ARG, "too many vertices");
        GarmentIn g;
        g.N = n;
        g.xyz.assign(cloth, cloth + 3 * (size_t)n);
        const int L = p.n_lists;
        g.rows.resize(L);
        g.ents.resize(L);
        g.ks.resize(L);
        for (int l = 0; l < L; ++l) {
            if (!rows[l]) return fail(VISG_ERR_INVALID_ARG, "csr_row[l] is NULL");
            g.rows[l].assign(rows[l], rows[l] + n + 1);
            if (g.rows[l][0] != 0) return fail(VISG_ERR_INVALID_ARG, "csr_row[l][0] must be 0");
            for (int i = 0; i < n; ++i)
                if (g.rows[l][i + 1] < g.rows[l][i]) return fail(VISG_ERR_INVALID_ARG, "csr_row not monotonic");
            uint32_t El = g.rows[l][n];
            if (El > 0 && !csr[l]) return fail(VISG_ERR_INVALID_ARG, "csr[l] is NULL");
            g.ents[l].assign(csr[l], csr[l] + El);
            for (auto& e : g.ents[l])
                if (e.end < 0 || e.end >= n) return fail(VISG_ERR_INVALID_ARG, "spring end out of range");
            if (list_k && list_k[l]) g.ks[l].assign(list_k[l], list_k[l] + El);
        }
        for (int k = 0; k < n_pinned; ++k) {
            if (pinned[k] >= (uint32_t)n) return fail(VISG_ERR_INVALID_ARG, "pinned index out of range");
            g.pinned.push_back(pinned[k]);
        }
        g.nv = nv;
        g.nt = nt;
        if (nt > 0) {
            g.bxyz.assign(body, body + 3 * (size_t)nv);
            if (bn) g.bnrm.assign(bn, bn + 3 * (size_t)nv);
            g.tris.assign(tris, tris + 3 * (size_t)nt);
            for (uint32_t t : g.tris)
                if (t >= (uint32_t)nv) return fail(VISG_ERR_INVALID_ARG, "triangle index out of range");
        }
        N += n;
        gin.push_back(std::move(g));
        if (gid) *gid = (int)gin.size() - 1;
        return VISG_OK;
    }

    int finalize() {
        split = p.split_collision ? 1 : 0;
        stage = p.stage_neighbours ? 1 : 0;
        if (finalized) return fail(VISG_ERR_STATE, "already finalized");
        if (gin.empty()) return fail(VISG_ERR_INVALID_ARG, "no garments");
        int dev = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
        CU(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        CU(cudaStreamCreateWithFlags(&cap2, cudaStreamNonBlocking));
        CU(cudaStreamCreateWithFlags(&run2, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&fork2, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&join2, cudaEventDisableTiming));
        CU(cudaHostAlloc((void**)&h_status, 16, cudaHostAllocDefault));
        G = (int)gin.size();
        const int L = p.n_lists;
        voff.assign(G + 1, 0);
        eoff.assign(G + 1, 0);
        for (int g = 0; g < G; ++g) {
            voff[g + 1] = voff[g] + gin[g].N;
            int64_t e = 0;
            for (int l = 0; l < L; ++l) e += gin[g].rows[l][gin[g].N];
            eoff[g + 1] = eoff[g] + e;
            for (int l = 0; l < L; ++l)
                if (!gin[g].ks[l].empty()) perk = true;
            if (gin[g].nt > 0) any_body = true;
        }
        E = eoff[G];
        if (E >= (int64_t)ROW_MASK) return fail(VISG_ERR_INVALID_ARG, "too many spring entries");
        // merged CSR
        h_rowp.assign(N + 1, 0);
        std::vector<uint2> ent(E > 0 ? E : 1);
        std::vector<float> kk;
        if (perk) kk.resize(E);
        merged_pos.resize(E);
        int64_t c = 0;
        for (int g = 0; g < G; ++g) {
            const GarmentIn& gi = gin[g];
            std::vector<int64_t> lbase(L, 0);
            for (int l = 1; l < L; ++l) lbase[l] = lbase[l - 1] + gi.rows[l - 1][gi.N];
            for (int i = 0; i < gi.N; ++i) {
                h_rowp[voff[g] + i] = (uint32_t)c;
                for (int l = 0; l < L; ++l) {
                    for (uint32_t e = gi.rows[l][i]; e < gi.rows[l][i + 1]; ++e) {
                        uint32_t j = (uint32_t)(voff[g] + gi.ents[l][e].end);
                        uint32_t rest;
                        std::memcpy(&rest, &gi.ents[l][e].rest, 4);
                        ent[c] = make_uint2(j | ((uint32_t)l << LIST_SHIFT), rest);
                        if (perk) kk[c] = gi.ks[l].empty() ? p.list_k[l] : gi.ks[l][e];
                        merged_pos[c] = eoff[g] + lbase[l] + e;
                        ++c;
                    }
                }
            }
            for (uint32_t v : gi.pinned) h_rowp[voff[g] + v] |= PIN_BIT;
        }
        h_rowp[N] = (uint32_t)E;
        // sliced ELL: slices of 32 vertices of one garment, each padded to its longest row
        std::vector<int64_t> slice0(G + 1, 0);
        for (int g = 0; g < G; ++g) slice0[g + 1] = slice0[g] + (gin[g].N + 31) / 32;
        const int64_t S = slice0[G];
        std::vector<uint32_t> soff(S + 1, 0);
        h_vcount.assign(N, make_uint2(0u, 0u));
        auto row_len = [&](int64_t v) { return (h_rowp[v + 1] & ROW_MASK) - (h_rowp[v] & ROW_MASK); };
        {
            uint64_t c2 = 0;
            for (int g = 0; g < G; ++g)
                for (int64_t s = slice0[g]; s < slice0[g + 1]; ++s) {
                    const int64_t v0 = voff[g] + 32 * (s - slice0[g]), v1 = std::min<int64_t>(v0 + 32, voff[g + 1]);
                    uint32_t w = 0;
                    for (int64_t v = v0; v < v1; ++v) w = std::max(w, row_len(v));
                    soff[s] = (uint32_t)c2;
                    c2 += 32ull * w;
                    if (c2 >= 0xffffffffull) return fail(VISG_ERR_INVALID_ARG, "too many spring entries");
                }
            soff[S] = (uint32_t)c2;
        }
        const int64_t ES = soff[S];
        std::vector<uint2> sell(ES > 0 ? ES : 1, make_uint2(0u, 0u));
        std::vector<float> sellk;
        if (perk) sellk.assign(ES > 0 ? ES : 1, 0.0f);
        for (int g = 0; g < G; ++g)
            for (int64_t v = voff[g]; v < voff[g + 1]; ++v) {
                const int64_t s = slice0[g] + (v - voff[g]) / 32;
                const int64_t lane = (v - voff[g]) % 32;
                const uint32_t rp = h_rowp[v] & ROW_MASK, n = row_len(v);
                uint32_t c[VISG_MAX_LISTS] = {0u, 0u, 0u, 0u};
                for (uint32_t k = 0; k < n; ++k) ++c[ent[rp + k].x >> LIST_SHIFT];
                if (c[0] > 0xffffu || c[1] > 0xffffu || c[2] > 0xffffu || c[3] > 0x7fffu)
                    return fail(VISG_ERR_UNSUPPORTED, "more than 65535 springs of one list at one vertex");
                h_vcount[v] = make_uint2(c[0] | (c[1] << 16), c[2] | (c[3] << 16) | (h_rowp[v] & PIN_BIT));
                for (uint32_t k = 0; k < n; ++k) {
                    sell[soff[s] + 32 * (int64_t)k + lane] = ent[rp + k];
                    if (perk) sellk[soff[s] + 32 * (int64_t)k + lane] = kk[rp + k];
                }
            }
        // tiles for each block size, with the sliced-ELL block of each one's slices
        std::vector<std::vector<int4>> tiles(kNumBlocks);
        std::vector<std::vector<int2>> twin(kNumBlocks);
        for (int b = 0; b < kNumBlocks; ++b) {
            const int cap = kStageCap[b];
            win_cap[b] = 0;
            for (int g = 0; g < G; ++g)
                for (int64_t v = voff[g]; v < voff[g + 1]; v += kBlocks[b]) {
                    const int64_t v1 = std::min<int64_t>(v + kBlocks[b], voff[g + 1]);
                    const int64_t s0 = slice0[g] + (v - voff[g]) / 32, s1 = s0 + (v1 - v + 31) / 32;
                    tiles[b].push_back(make_int4(g | (gin[g].nt > 0 ? TILE_BODY : 0), (int)v, (int)v1, (int)s0));
                    const int64_t cnt = (int64_t)soff[s1] - soff[s0];
                    if (cnt > 0 && cnt <= cap && soff[s1] <= 0x7fffffffu) {
                        twin[b].push_back(make_int2((int)soff[s0], (int)cnt));
                        win_cap[b] = std::max(win_cap[b], (int)cnt);
                    } else {
                        twin[b].push_back(make_int2(0, 0));
                    }
                }
        }
        // the two garment groups: split at the garment boundary nearest half the vertices
        if (G >= 2) {
            int gs = 1;
            for (int g = 2; g < G; ++g)
                if (std::llabs(2 * voff[g] - N) < std::llabs(2 * voff[gs] - N)) gs = g;
            vsplit = voff[gs];
            for (int b = 0; b < kNumBlocks; ++b) {
                tsplit[b] = 0;
                while (tsplit[b] < (int)tiles[b].size() && (tiles[b][tsplit[b]].x & TILE_GARMENT) < gs) ++tsplit[b];
            }
        }
        // plan the allocation
        arena.want(&d_state[0], 2 * (size_t)N + 2);
        arena.want(&d_state[1], 2 * (size_t)N + 2);
        arena.want(&d_normal, (size_t)N + 1);
        arena.want(&d_rowp, (size_t)N + 2);
        arena.want(&d_ent, (size_t)E + 1);
        if (perk) arena.want(&d_k, (size_t)E + 1);
        for (int b = 0; b < kNumBlocks; ++b) {
            n_tiles[b] = (int)tiles[b].size();
            arena.want(&d_tiles[b], tiles[b].size() + 1);
            arena.want(&d_twin[b], twin[b].size() + 1);
        }
        arena.want(&d_sell, sell.size());
        if (perk) arena.want(&d_sellk, sellk.size());
        arena.want(&d_slice_off, soff.size());
        arena.want(&d_vcount, h_vcount.size());
        arena.want(&d_wild, 4);
        arena.want(&d_views, (size_t)G);
        arena.want(&d_err, 4);
        arena.want(&d_check, 4);
        arena.want(&d_cand, (size_t)N + 1);
        arena.want(&d_cand_count, 4);
        arena.want(&d_stage, 10 * (size_t)N + 4);
        bvh.resize(G);
        for (int g = 0; g < G; ++g)
            if (gin[g].nt > 0) {
                bvh[g].plan(arena, gin[g].nv, gin[g].nt, !gin[g].bnrm.empty());
                bvh[g].coherent = true;  // rebuilt in place: the last build's order is at hand
            }
        CU(arena.commit());
        // upload
        std::vector<float4> st(2 * (size_t)N);
        float xo_is_x_bits;
        const uint32_t fl0 = FLAG_XO_IS_X;
        std::memcpy(&xo_is_x_bits, &fl0, 4);
        for (int g = 0; g < G; ++g)
            for (int i = 0; i < gin[g].N; ++i) {
                const float* q = &gin[g].xyz[3 * (size_t)i];
                int64_t v = voff[g] + i;
                st[2 * v] = make_float4(q[0], q[1], q[2], 0.0f);  // x = x_old: v = 0 (simulation.cu:84-85)
                st[2 * v + 1] = make_float4(0.0f, 0.0f, xo_is_x_bits, 0.0f);
            }
        CU(cudaMemcpy(d_state[0], st.data(), st.size() * sizeof(float4), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_rowp, h_rowp.data(), h_rowp.size() * 4, cudaMemcpyHostToDevice));
        if (E > 0) CU(cudaMemcpy(d_ent, ent.data(), E * sizeof(uint2), cudaMemcpyHostToDevice));
        if (perk && E > 0) CU(cudaMemcpy(d_k, kk.data(), E * sizeof(float), cudaMemcpyHostToDevice));
        for (int b = 0; b < kNumBlocks; ++b) {
            CU(cudaMemcpy(d_tiles[b], tiles[b].data(), tiles[b].size() * sizeof(int4), cudaMemcpyHostToDevice));
            CU(cudaMemcpy(d_twin[b], twin[b].data(), twin[b].size() * sizeof(int2), cudaMemcpyHostToDevice));
        }
        CU(cudaMemcpy(d_sell, sell.data(), sell.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        if (perk) CU(cudaMemcpy(d_sellk, sellk.data(), sellk.size() * sizeof(float), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_slice_off, soff.data(), soff.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_vcount, h_vcount.data(), h_vcount.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        CU(cudaMemsetAsync(d_wild, 0, 4, stream));
        CU(launch_check_tame(d_state[0], N, d_wild, stream));
        std::vector<BvhView> views(G);
        for (int g = 0; g < G; ++g)
            views[g] = gin[g].nt > 0 ? bvh[g].view() : BvhView{nullptr, nullptr, nullptr};
        CU(cudaMemcpy(d_views, views.data(), G * sizeof(BvhView), cudaMemcpyHostToDevice));
        for (int g = 0; g < G; ++g) {
            if (gin[g].nt == 0) continue;
            CU(cudaMemcpy(bvh[g].xyz_in, gin[g].bxyz.data(), gin[g].bxyz.size() * 4, cudaMemcpyHostToDevice));
            if (!gin[g].bnrm.empty())
                CU(cudaMemcpy(bvh[g].nrm_in, gin[g].bnrm.data(), gin[g].bnrm.size() * 4, cudaMemcpyHostToDevice));
            CU(cudaMemcpy(bvh[g].tris, gin[g].tris.data(), gin[g].tris.size() * 4, cudaMemcpyHostToDevice));
            CU(lbvh_build(bvh[g], p.thickness, p.box_depth, d_err, stream));
        }
        // keep only what later calls need
        for (auto& g : gin) {
            std::vector<float>().swap(g.xyz);
            std::vector<float>().swap(g.bxyz);
            std::vector<float>().swap(g.bnrm);
            std::vector<uint32_t>().swap(g.tris);
        }
        finalized = true;
        return sync();
    }

    int variant(int blk) const {
        int v = variant();
        const int bi = block_index(blk);
        if (stage && bi >= 0 && win_cap[bi] > 0) v |= SV_STAGED;
        return v;
    }

    int variant() const {  // without the launch-shape dependent bits
        int v = 0;
        if (perk) v |= SV_PERK;
        if (p.verlet_damping == 1.0f) v |= SV_REFV;
        if (p.collide && any_body) v |= SV_COLLIDE;
        if (p.collide && any_body && split) v |= SV_SPLIT;
        if (p.check_every > 0) v |= SV_CHECK;
        uint32_t kdbits;
        std::memcpy(&kdbits, &p.spring_damping, 4);
        if (kdbits == 0u) v |= SV_KD0;
        return v;
    }

    StepParams step_params() const {
        StepParams sp;
        sp.dt = p.dt;
        sp.mass = p.mass;
        sp.gx = p.gravity[0];
        sp.gy = p.gravity[1];
        sp.gz = p.gravity[2];
        sp.damp = p.force_damping;
        sp.kd = p.spring_damping;
        sp.gamma = p.verlet_damping;
        for (int l = 0; l < VISG_MAX_LISTS; ++l) sp.list_k[l] = p.list_k[l];
        sp.n_lists = p.n_lists;
        sp.max_disp = p.max_displacement;
        sp.margin = p.collision_margin ? 1 : 0;
        uint32_t kdb;
        std::memcpy(&kdb, &p.spring_damping, 4);
        sp.drec = (kdb == 0u && p.verlet_damping != 1.0f && p.n_lists >= 1) ? 1 : 0;
        sp.dmax = 0.5e15f * p.dt;
        return sp;
    }

    // step chains per step: two garment groups, or one
    int groups() const { return (G >= 2 && p.overlap_groups != 1) ? 2 : 1; }

    StepArgs args(int from, int blk, int grp = 0) const {
        StepArgs a;
        a.state_in = d_state[from];
        a.state_out = d_state[from ^ 1];
        a.normal = d_normal;
        a.rowp = d_rowp;
        a.ent = d_ent;
        a.kent = d_k;
        int bi = block_index(blk);
        const int two = groups() == 2;
        const int t0 = (two && grp == 1) ? tsplit[bi] : 0, t1 = (two && grp == 0) ? tsplit[bi] : n_tiles[bi];
        a.tiles = d_tiles[bi] + t0;
        a.n_tiles = t1 - t0;
        a.bodies = d_views;
        a.err = d_err;
        a.check = d_check;
        a.cand = d_cand + ((two && grp == 1) ? vsplit : 0);  // a group queues at most its own vertices
        a.cand_count = d_cand_count + ((two && grp == 1) ? 1 : 0);
        a.sell = d_sell;
        a.sellk = d_sellk;
        a.slice_off = d_slice_off;
        a.vcount = d_vcount;
        a.wild = d_wild;
        a.twin = d_twin[bi] + t0;
        a.win_cap = win_cap[bi];
        a.p = step_params();
        return a;
    }

    // the step kernel's grid: with two overlapping chains and persistent CTAs, `reserve`
    // SMs' worth of CTAs fewer
    int step_grid() const {
        if (groups() != 2 || grid <= 0 || reserve <= 0 || sm_count <= reserve) return grid;
        return (grid / sm_count) * (sm_count - reserve);
    }

    // one step; with two groups the second runs on its own stream (forked from and
    // joined back to s) so the two chains overlap as they do in the step graphs
    cudaError_t launch_one(cudaStream_t s, int from) {
        if (groups() == 1) return launch_step(args(from, block, 0), variant(block), block, grid, s);
        cudaError_t e = cudaEventRecord(fork2, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(run2, fork2, 0);
        if (e == cudaSuccess) e = launch_step(args(from, block, 1), variant(block), block, step_grid(), run2);
        cudaError_t e0 = launch_step(args(from, block, 0), variant(block), block, step_grid(), s);
        cudaError_t ej = cudaEventRecord(join2, run2);
        if (ej == cudaSuccess) ej = cudaStreamWaitEvent(s, join2, 0);
        return e != cudaSuccess ? e : (e0 != cudaSuccess ? e0 : ej);
    }

    // chunk_steps steps as one graph; with two groups each group's steps form their own
    // chain on its own capture stream (forked at the start, joined at the end), so
    // the chains overlap when the graph runs
    int capture_chunk(int c) {
        cudaGraph_t g = nullptr;
        const int ng = groups();
        CU(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        cudaError_t le = cudaSuccess;
        if (ng == 2) {
            le = cudaEventRecord(fork_ev, cap);
            if (le == cudaSuccess) le = cudaStreamWaitEvent(cap2, fork_ev, 0);
        }
        int from = c;
        for (int k = 0; k < chunk_steps && le == cudaSuccess; ++k) {
            for (int gr = 0; gr < ng; ++gr) {
                cudaError_t e = launch_step(args(from, block, gr), variant(block), block, step_grid(), gr ? cap2 : cap);
                if (e != cudaSuccess && le == cudaSuccess) le = e;
            }
            from ^= 1;
        }
        if (ng == 2) {  // join, even after an error, so the capture can end
            cudaError_t e = cudaEventRecord(join_ev, cap2);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(cap, join_ev, 0);
            if (e != cudaSuccess && le == cudaSuccess) le = e;
        }
        cudaError_t ee = cudaStreamEndCapture(cap, &g);
        if (le != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(le, "step capture");
        }
        CU(ee);
        cudaError_t ie = cudaGraphInstantiate(&chunk_exec[c], g, 0);
        cudaGraphDestroy(g);
        CU(ie);
        return VISG_OK;
    }

    int step(int n) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (n < 0) return fail(VISG_ERR_INVALID_ARG, "nsteps < 0");
        if (n > 0) prev_ok = true;
        while (n > 0) {
            if (p.use_graph && n >= chunk_steps) {
                if (!chunk_exec[cur]) {
                    int r = capture_chunk(cur);
                    if (r) return r;
                }
                CU(cudaGraphLaunch(chunk_exec[cur], stream));
                n -= chunk_steps;
                steps_since_check += chunk_steps;
            } else {
                CU(launch_one(stream, cur));
                cur ^= 1;
                --n;
                ++steps_since_check;
            }
            if (p.check_every > 0 && steps_since_check >= p.check_every) {
                steps_since_check = 0;
                int r = sync();
                if (r) return r;
            }
        }
        return VISG_OK;
    }

    // n steps as one chain (each launch covers the whole batch), with CUDA events right
    // around each step-kernel launch and after each collision pass on the step stream:
    // the average device time per launch of each kernel
    int time_kernels(int n, float* ms_step, float* ms_collide) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (n <= 0 || !ms_step) return fail(VISG_ERR_INVALID_ARG, "nsteps <= 0 or ms_step is NULL");
        cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
        for (auto& x : ev) CU(cudaEventCreate(&x));
        const int saved = p.overlap_groups;
        p.overlap_groups = 1;
        double ts = 0.0, tc = 0.0;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < n && e == cudaSuccess; ++k) {
            set_step_timing(ev[0], ev[1]);
            e = launch_step(args(cur, block, 0), variant(block), block, grid, stream);
            set_step_timing(nullptr, nullptr);
            if (e == cudaSuccess) e = cudaEventRecord(ev[2], stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[2]);
            float a = 0.0f, b = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&a, ev[0], ev[1]);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&b, ev[1], ev[2]);
            ts += a;
            tc += b;
            cur ^= 1;
        }
        p.overlap_groups = saved;
        prev_ok = true;
        for (auto& x : ev) cudaEventDestroy(x);
        if (e != cudaSuccess) return cuda_fail(e, "kernel timing");
        *ms_step = (float)(ts / n);
        if (ms_collide) *ms_collide = (variant(block) & SV_SPLIT) ? (float)(tc / n) : 0.0f;
        return sync();
    }

    // wait, then report device-side errors (and the divergence check)
    int sync() {
        CU(cudaMemcpyAsync(h_status, d_err, 4, cudaMemcpyDeviceToHost, stream));
        CU(cudaMemcpyAsync(h_status + 1, d_check, 8, cudaMemcpyDeviceToHost, stream));
        CU(cudaStreamSynchronize(stream));
        uint32_t err = h_status[0];
        float maxd;
        std::memcpy(&maxd, &h_status[1], 4);
        uint32_t bad = h_status[2];
        if (err || bad || (p.check_every > 0 && maxd > p.max_displacement)) {
            CU(cudaMemsetAsync(d_err, 0, 4, stream));
            CU(cudaMemsetAsync(d_check, 0, 8, stream));
            CU(cudaStreamSynchronize(stream));
            if (err & ERR_TIMEOUT) return fail(VISG_ERR_TIMEOUT, "a bounded device wait gave up (LBVH look-back or step stage copy)");
            if (err & ERR_STACK) return fail(VISG_ERR_UNSUPPORTED, "BVH deeper than the traversal stack");
            if (err & ERR_INDEX) return fail(VISG_ERR_INVALID_ARG, "an index read on the device was out of range");
            char buf[160];
            std::snprintf(buf, sizeof buf, "diverged: %u non-finite vertices, max step displacement %g (limit %g)", bad,
                          (double)maxd, (double)p.max_displacement);
            return fail(VISG_ERR_DIVERGED, buf);
        }
        if (p.check_every > 0) CU(cudaMemsetAsync(d_check, 0, 8, stream));
        return VISG_OK;
    }

    int update_body(int g, const float* xyz, const float* nrm, cudaMemcpyKind kind) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (g < 0 || g >= G) return fail(VISG_ERR_INVALID_ARG, "garment out of range");
        if (gin[g].nt == 0) return fail(VISG_ERR_STATE, "garment has no body");
        if (!xyz) return fail(VISG_ERR_INVALID_ARG, "body_xyz is NULL");
        if ((nrm != nullptr) != bvh[g].has_normals)
            return fail(VISG_ERR_INVALID_ARG, "body normals must be given iff they were given at creation");
        // device arrays are read by the build itself, in stream order; host arrays are
        // staged first.  The build also voids the garment's query-cache margins (the
        // body moves)
        const bool dev = kind == cudaMemcpyDeviceToDevice;
        if (!dev) {
            CU(cudaMemcpyAsync(bvh[g].xyz_in, xyz, (size_t)bvh[g].nv * 12, kind, stream));
            if (nrm) CU(cudaMemcpyAsync(bvh[g].nrm_in, nrm, (size_t)bvh[g].nv * 12, kind, stream));
        }
        CU(lbvh_build(bvh[g], p.thickness, p.box_depth, d_err, stream, dev ? xyz : nullptr, dev ? nrm : nullptr,
                      d_state[cur], voff[g], voff[g + 1]));
        return VISG_OK;
    }

    int check_vertex(int g, uint32_t idx, int64_t* v) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (g < 0 || g >= G) return fail(VISG_ERR_INVALID_ARG, "garment out of range");
        if (idx >= (uint32_t)gin[g].N) return fail(VISG_ERR_INVALID_ARG, "vertex index out of range");
        *v = voff[g] + idx;
        return VISG_OK;
    }

    int set_vertex(int g, uint32_t idx, const float* xyz) {
        int64_t v = 0;
        if (int r = check_vertex(g, idx, &v)) return r;
        if (!xyz) return fail(VISG_ERR_INVALID_ARG, "xyz is NULL");
        const uint32_t gi = (uint32_t)v;  // x and x_old (simulation.cu:255-256)
        if (int r = set_vertices(&gi, xyz, 1)) return r;
        CU(cudaStreamSynchronize(stream));
        return VISG_OK;
    }

    // many vertices at once: host arrays staged into a pinned buffer, one H2D, one scatter
    uint32_t* d_sv_idx = nullptr;
    float* d_sv_xyz = nullptr;
    char* h_sv = nullptr;
    int sv_cap = 0;
    cudaEvent_t sv_done = nullptr;
    int set_vertices(const uint32_t* idx, const float* xyz, int n) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (n < 0 || (n > 0 && (!idx || !xyz))) return fail(VISG_ERR_INVALID_ARG, "bad vertex list");
        for (int k = 0; k < n; ++k)
            if (idx[k] >= (uint64_t)N) return fail(VISG_ERR_INVALID_ARG, "vertex index out of range");
        if (n == 0) return VISG_OK;
        if (n > sv_cap) {
            if (sv_done) CU(cudaEventSynchronize(sv_done));
            cudaFree(d_sv_idx);
            cudaFreeHost(h_sv);
            d_sv_idx = nullptr;
            h_sv = nullptr;
            int cap = std::max(n, 1024);
            CU(cudaMalloc((void**)&d_sv_idx, (size_t)cap * 16));
            d_sv_xyz = (float*)(d_sv_idx + cap);
            CU(cudaHostAlloc((void**)&h_sv, (size_t)cap * 16, cudaHostAllocDefault));
            if (!sv_done) CU(cudaEventCreateWithFlags(&sv_done, cudaEventDisableTiming));
            sv_cap = cap;
        }
        CU(cudaEventSynchronize(sv_done));  // the previous upload has left the staging buffer
        std::memcpy(h_sv, idx, (size_t)n * 4);
        std::memcpy(h_sv + (size_t)sv_cap * 4, xyz, (size_t)n * 12);
        CU(cudaMemcpyAsync(d_sv_idx, h_sv, (size_t)n * 4, cudaMemcpyHostToDevice, stream));
        CU(cudaMemcpyAsync(d_sv_xyz, h_sv + (size_t)sv_cap * 4, (size_t)n * 12, cudaMemcpyHostToDevice, stream));
        CU(cudaEventRecord(sv_done, stream));
        CU(launch_set_vertices(d_state[cur], d_sv_idx, d_sv_xyz, n, p.dt, d_wild, stream));
        return VISG_OK;
    }

    int set_pinned(const uint32_t* idx, int n) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (n < 0 || (n > 0 && !idx)) return fail(VISG_ERR_INVALID_ARG, "bad pin list");
        for (int k = 0; k < n; ++k)
            if (idx[k] >= (uint32_t)N) return fail(VISG_ERR_INVALID_ARG, "pinned index out of range");
        for (int64_t i = 0; i < N; ++i) h_rowp[i] &= ROW_MASK;
        for (int k = 0; k < n; ++k) h_rowp[idx[k]] |= PIN_BIT;
        for (int64_t i = 0; i < N; ++i) h_vcount[i].y = (h_vcount[i].y & ROW_MASK) | (h_rowp[i] & PIN_BIT);
        CU(cudaMemcpyAsync(d_rowp, h_rowp.data(), (size_t)N * 4, cudaMemcpyHostToDevice, stream));
        CU(cudaMemcpyAsync(d_vcount, h_vcount.data(), (size_t)N * sizeof(uint2), cudaMemcpyHostToDevice, stream));
        CU(cudaStreamSynchronize(stream));
        return VISG_OK;
    }

    // Enqueue, behind the steps issued so far, the read of all positions into host
    // memory `out`; returns at once.  The unpack runs on the step stream, the copy on
    // the read-back stream, so the steps issued next overlap the transfer.
    int read_positions_async(float* out) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (!out) return fail(VISG_ERR_INVALID_ARG, "out is NULL");
        if (rb.pending == kReadSlots) return fail(VISG_ERR_STATE, "three reads are in flight: wait for one first");
        if (!rb.copy) {
            CU(cudaStreamCreateWithFlags(&rb.copy, cudaStreamNonBlocking));
            CU(cudaHostAlloc((void**)&rb.h_err, 4 * kReadSlots, cudaHostAllocDefault));
            for (int k = 0; k < kReadSlots; ++k) {
                CU(cudaMalloc((void**)&rb.d_pos[k], (size_t)N * 12 + 16));
                CU(cudaEventCreateWithFlags(&rb.unpacked[k], cudaEventDisableTiming));
                CU(cudaEventCreateWithFlags(&rb.copied[k], cudaEventDisableTiming));
            }
        }
        const int k = rb.next;
        if (rb.used[k]) CU(cudaStreamWaitEvent(stream, rb.copied[k], 0));  // slot's last copy has left
        CU(launch_unpack_positions(d_state[cur], N, rb.d_pos[k], stream));
        CU(cudaMemcpyAsync(rb.h_err + k, d_err, 4, cudaMemcpyDeviceToHost, stream));
        CU(cudaEventRecord(rb.unpacked[k], stream));
        CU(cudaStreamWaitEvent(rb.copy, rb.unpacked[k], 0));
        CU(cudaMemcpyAsync(out, rb.d_pos[k], (size_t)N * 12, cudaMemcpyDeviceToHost, rb.copy));
        CU(cudaEventRecord(rb.copied[k], rb.copy));
        rb.used[k] = true;
        rb.next = (rb.next + 1) % kReadSlots;
        ++rb.pending;
        return VISG_OK;
    }

    // wait for the oldest read in flight; reports device-side errors like a sync
    int wait_positions() {
        if (rb.pending == 0) return fail(VISG_ERR_STATE, "no read in flight");
        const int k = (rb.next - rb.pending + kReadSlots) % kReadSlots;  // the oldest
        --rb.pending;
        CU(cudaEventSynchronize(rb.copied[k]));
        if (rb.h_err[k] != 0u) return sync();  // a device-side error: report it (and clear it)
        return VISG_OK;
    }

    void free_faces() {
        void* ps[] = {d_faces, d_frow, d_fcol, d_fnorm};
        for (void* q : ps)
            if (q) cudaFree(q);
        d_faces = d_frow = d_fcol = nullptr;
        d_fnorm = nullptr;
        NF = 0;
    }

    // faces of garment g (local vertex indices); rebuilds the device face arrays and
    // the vertex -> face CSR (get_vertex_adjface, simulation.cu:152-180: each vertex's
    // faces in face order)
    int set_faces(int g, const uint32_t* faces, int nf) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (g < 0 || g >= G) return fail(VISG_ERR_INVALID_ARG, "garment out of range");
        if (nf < 0 || (nf > 0 && !faces)) return fail(VISG_ERR_INVALID_ARG, "faces is NULL or n_faces < 0");
        const int64_t ng = voff[g + 1] - voff[g];
        for (int64_t k = 0; k < 3 * (int64_t)nf; ++k)
            if (faces[k] >= (uint64_t)ng) return fail(VISG_ERR_INVALID_ARG, "face vertex index out of range");
        if (int r = sync()) return r;
        gfaces.resize(G);
        gfaces[g].assign(faces, faces + 3 * (size_t)nf);
        int64_t nft = 0;
        for (auto& f : gfaces) nft += (int64_t)f.size() / 3;
        if (3 * nft >= (int64_t)0xffffffffu) return fail(VISG_ERR_INVALID_ARG, "too many faces");
        std::vector<uint32_t> hf(3 * (size_t)nft + 3), row(N + 1, 0), col(3 * (size_t)nft + 1);
        int64_t fo = 0;
        for (int gg = 0; gg < G; ++gg) {
            for (size_t k = 0; k < gfaces[gg].size(); ++k) hf[3 * fo + k] = (uint32_t)(voff[gg] + gfaces[gg][k]);
            fo += (int64_t)gfaces[gg].size() / 3;
        }
        for (int64_t k = 0; k < 3 * nft; ++k) ++row[hf[k] + 1];
        for (int64_t v = 0; v < N; ++v) row[v + 1] += row[v];
        std::vector<uint32_t> fill(row.begin(), row.end() - 1);
        for (int64_t f = 0; f < nft; ++f)
            for (int j = 0; j < 3; ++j) col[fill[hf[3 * f + j]]++] = (uint32_t)f;
        free_faces();
        CU(cudaMalloc((void**)&d_faces, hf.size() * 4));
        CU(cudaMalloc((void**)&d_frow, row.size() * 4));
        CU(cudaMalloc((void**)&d_fcol, col.size() * 4));
        CU(cudaMalloc((void**)&d_fnorm, (3 * (size_t)nft + 3) * 4));
        CU(cudaMemcpy(d_faces, hf.data(), hf.size() * 4, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_frow, row.data(), row.size() * 4, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d_fcol, col.data(), col.size() * 4, cudaMemcpyHostToDevice));
        NF = nft;
        return VISG_OK;
    }

    // the output stage of cuda_update_vbo (simulation.cu:196-231) into caller buffers:
    // pos4 (N x 4), vertex normals (N x 3), face normals (F x 3); any may be NULL.
    // Normals are of the positions the last step started from (the reference's
    // choice) when `prev` is set and a step has run, else of the current positions.
    int render(float* pos4, float* vn, float* fn, float* colour, const float* rgb, int on_device, int prev) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if ((vn || fn || colour) && !d_frow) return fail(VISG_ERR_STATE, "normals need the faces (visg_set_faces)");
        if (colour && !rgb) return fail(VISG_ERR_INVALID_ARG, "shaded colours need the object colour");
        const float4* now = d_state[cur];
        const float4* from = (prev && prev_ok) ? d_state[cur ^ 1] : d_state[cur];
        float4* dpos = on_device ? (float4*)pos4 : (pos4 ? (float4*)d_stage : nullptr);
        float* dvn = on_device ? vn : (vn ? d_stage + 4 * N : nullptr);
        float* dcol = on_device ? colour : (colour ? d_stage + 7 * N : nullptr);
        float* dfn = (on_device && fn) ? fn : d_fnorm;
        CU(launch_render(now, from, N, d_faces, NF, d_frow, d_fcol, (vn || fn || colour) ? dfn : nullptr, dpos, dvn,
                         dcol, rgb, stream));
        if (on_device) return VISG_OK;
        if (pos4) CU(cudaMemcpyAsync(pos4, d_stage, (size_t)N * 16, cudaMemcpyDeviceToHost, stream));
        if (vn) CU(cudaMemcpyAsync(vn, d_stage + 4 * N, (size_t)N * 12, cudaMemcpyDeviceToHost, stream));
        if (colour) CU(cudaMemcpyAsync(colour, d_stage + 7 * N, (size_t)N * 12, cudaMemcpyDeviceToHost, stream));
        if (fn && NF > 0) CU(cudaMemcpyAsync(fn, d_fnorm, (size_t)NF * 12, cudaMemcpyDeviceToHost, stream));
        return sync();
    }

    int get_positions(int g, float* out, int on_device) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (!out) return fail(VISG_ERR_INVALID_ARG, "out is NULL");
        int64_t v0 = 0, n = N;
        if (g >= 0) {
            if (g >= G) return fail(VISG_ERR_INVALID_ARG, "garment out of range");
            v0 = voff[g];
            n = voff[g + 1] - voff[g];
        }
        if (on_device) {
            CU(launch_unpack_positions(d_state[cur] + 2 * v0, n, out, stream));
            return VISG_OK;
        }
        CU(launch_unpack_positions(d_state[cur] + 2 * v0, n, d_stage, stream));
        CU(cudaMemcpyAsync(out, d_stage, (size_t)n * 12, cudaMemcpyDeviceToHost, stream));
        return sync();
    }

    int count_contacts(int64_t* out) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (!out) return fail(VISG_ERR_INVALID_ARG, "out is NULL");
        unsigned long long* d = (unsigned long long*)d_stage;
        CU(cudaMemsetAsync(d, 0, 8, stream));
        CU(launch_count_contacts(d_state[cur], N, d, stream));
        unsigned long long h = 0;
        CU(cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, stream));
        CU(cudaStreamSynchronize(stream));
        *out = (int64_t)h;
        return sync();
    }

    // vertex range of garment g (g = -1: all garments)
    int garment_range(int g, int64_t& v0, int64_t& n) const {
        v0 = 0;
        n = N;
        if (g < 0) return VISG_OK;
        if (g >= G) return fail(VISG_ERR_INVALID_ARG, "garment out of range");
        v0 = voff[g];
        n = voff[g + 1] - voff[g];
        return VISG_OK;
    }

    int get_state(int g, float* x, float* xo, float* nrm) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        int64_t v0, n;
        if (int r = garment_range(g, v0, n)) return r;
        float* sx = d_stage;
        float* sxo = d_stage + 3 * n;
        float* sn = d_stage + 6 * n;
        CU(launch_unpack_state(d_state[cur] + 2 * v0, d_state[cur ^ 1] + 2 * v0, d_normal + v0, n, sx, sxo, sn,
                               stream));
        if (x) CU(cudaMemcpyAsync(x, sx, (size_t)n * 12, cudaMemcpyDeviceToHost, stream));
        if (xo) CU(cudaMemcpyAsync(xo, sxo, (size_t)n * 12, cudaMemcpyDeviceToHost, stream));
        if (nrm) CU(cudaMemcpyAsync(nrm, sn, (size_t)n * 12, cudaMemcpyDeviceToHost, stream));
        return sync();
    }

    int set_state(int g, const float* x, const float* xo, const float* nrm) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        int64_t v0, n;
        if (int r = garment_range(g, v0, n)) return r;
        float* sx = d_stage;
        float* sxo = d_stage + 3 * n;
        float* sn = d_stage + 6 * n;
        if (x) CU(cudaMemcpyAsync(sx, x, (size_t)n * 12, cudaMemcpyHostToDevice, stream));
        if (xo) CU(cudaMemcpyAsync(sxo, xo, (size_t)n * 12, cudaMemcpyHostToDevice, stream));
        if (nrm) CU(cudaMemcpyAsync(sn, nrm, (size_t)n * 12, cudaMemcpyHostToDevice, stream));
        prev_ok = false;
        CU(launch_pack_state(d_state[cur] + 2 * v0, d_state[cur ^ 1] + 2 * v0, d_normal + v0, n, x ? sx : nullptr,
                             xo ? sxo : nullptr, nrm ? sn : nullptr, p.dt, step_params().drec,
                             step_params().dmax, d_wild, stream));
        CU(cudaStreamSynchronize(stream));
        return VISG_OK;
    }

    int export_lbvh(int g, uint32_t* tri_codes, float* tri_boxes, uint32_t* sorted_codes, int32_t* sorted_tris,
                    int32_t* child_a, int32_t* child_b, int32_t* parent_int, int32_t* parent_leaf, float* int_boxes,
                    float* leaf_boxes, float* root_box) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (int r = sync()) return r;
        const BvhBuffers& b = bvh[g];
        const int T = gin[g].nt;
        if (T == 0) return VISG_OK;
        BvhRoot rt;
        CU(cudaMemcpy(&rt, b.root, sizeof rt, cudaMemcpyDeviceToHost));
        const int Tp = rt.n_leaves;
        std::vector<uint32_t> codes(T), ucode(Tp), utri(Tp);
        std::vector<float4> tb(2 * (size_t)T);
        CU(cudaMemcpy(codes.data(), b.codes, T * 4, cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(tb.data(), b.tri_box, tb.size() * sizeof(float4), cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(ucode.data(), b.ucode, Tp * 4, cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(utri.data(), b.utri, Tp * 4, cudaMemcpyDeviceToHost));
        auto put = [](float* dst, float4 lo, float4 hi) {
            dst[0] = lo.x; dst[1] = lo.y; dst[2] = lo.z; dst[3] = hi.x; dst[4] = hi.y; dst[5] = hi.z;
        };
        for (int t = 0; t < T; ++t) {
            if (tri_codes) tri_codes[t] = codes[t];
            if (tri_boxes) put(tri_boxes + 6 * t, tb[2 * t], tb[2 * t + 1]);
        }
        for (int i = 0; i < Tp; ++i) {
            if (sorted_codes) sorted_codes[i] = ucode[i];
            if (sorted_tris) sorted_tris[i] = (int32_t)utri[i];
        }
        if (root_box) put(root_box, rt.frame_lo, rt.frame_hi);
        if (Tp == 1) {
            if (parent_leaf) parent_leaf[0] = 0;
            if (leaf_boxes) put(leaf_boxes, rt.top_lo, rt.top_hi);
            return VISG_OK;
        }
        const int ni = Tp - 1;
        std::vector<Node> nd(ni);
        std::vector<int2> rg(ni);
        CU(cudaMemcpy(nd.data(), b.nodes, ni * sizeof(Node), cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(rg.data(), b.range, ni * sizeof(int2), cudaMemcpyDeviceToHost));
        // renumber split-indexed nodes into the reference's layout: the root is 0, an
        // internal node that is child A has the index of its last leaf, child B of its first
        std::vector<int> kidx(ni, -1);
        kidx[rt.root] = 0;
        auto link = [](float w) {
            int v;
            std::memcpy(&v, &w, 4);
            return v;
        };
        for (int gg = 0; gg < ni; ++gg) {
            int la = link(nd[gg].a_lo.w), lb = link(nd[gg].b_lo.w);
            if (la >= 0) kidx[la] = rg[la].y;
            if (lb >= 0) kidx[lb] = rg[lb].x;
        }
        for (int gg = 0; gg < ni; ++gg)
            if (kidx[gg] < 0 || kidx[gg] >= ni) return fail(VISG_ERR_CUDA, "LBVH export: inconsistent tree");
        std::vector<int32_t> ca(ni, 0), cb(ni, 0), pi(ni, 0), pl(Tp, 0);
        std::vector<float> ib(6 * (size_t)ni, 0.0f), lb6(6 * (size_t)Tp, 0.0f);
        put(&ib[0], rt.top_lo, rt.top_hi);  // root box (identity U A U B)
        for (int gg = 0; gg < ni; ++gg) {
            const int k = kidx[gg];
            const int la = link(nd[gg].a_lo.w), lbk = link(nd[gg].b_lo.w);
            if (la < 0) {
                ca[k] = -(~la) - 1;
                pl[~la] = k + 1;
                put(&lb6[6 * (size_t)(~la)], nd[gg].a_lo, nd[gg].a_hi);
            } else {
                ca[k] = kidx[la] + 1;
                pi[kidx[la]] = k + 1;
                put(&ib[6 * (size_t)kidx[la]], nd[gg].a_lo, nd[gg].a_hi);
            }
            if (lbk < 0) {
                cb[k] = -(~lbk) - 1;
                pl[~lbk] = k + 1;
                put(&lb6[6 * (size_t)(~lbk)], nd[gg].b_lo, nd[gg].b_hi);
            } else {
                cb[k] = kidx[lbk] + 1;
                pi[kidx[lbk]] = k + 1;
                put(&ib[6 * (size_t)kidx[lbk]], nd[gg].b_lo, nd[gg].b_hi);
            }
        }
        if (child_a) std::memcpy(child_a, ca.data(), ni * 4);
        if (child_b) std::memcpy(child_b, cb.data(), ni * 4);
        if (parent_int) std::memcpy(parent_int, pi.data(), ni * 4);
        if (parent_leaf) std::memcpy(parent_leaf, pl.data(), Tp * 4);
        if (int_boxes) std::memcpy(int_boxes, ib.data(), ib.size() * 4);
        if (leaf_boxes) std::memcpy(leaf_boxes, lb6.data(), lb6.size() * 4);
        return VISG_OK;
    }

    int query(int g, const float* pts, int n, int32_t* leaf, int32_t* inside, float* dist, float* normal) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (n < 0 || (n > 0 && !pts)) return fail(VISG_ERR_INVALID_ARG, "bad points");
        if (n == 0) return VISG_OK;
        if (gin[g].nt == 0) {
            for (int i = 0; i < n; ++i) {
                if (leaf) leaf[i] = -1;
                if (inside) inside[i] = 0;
                if (dist) dist[i] = 0.0f;
                if (normal) normal[3 * i] = normal[3 * i + 1] = normal[3 * i + 2] = 0.0f;
            }
            return VISG_OK;
        }
        char* buf = nullptr;
        size_t bytes = (size_t)n * (12 + 4 + 4 + 4 + 12);
        CU(cudaMalloc((void**)&buf, bytes));
        float* dp = (float*)buf;
        int* dl = (int*)(dp + 3 * (size_t)n);
        int* di = dl + n;
        float* dd = (float*)(di + n);
        float* dn = dd + n;
        cudaError_t e = cudaMemcpyAsync(dp, pts, (size_t)n * 12, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = launch_query(bvh[g].view(), dp, n, dl, di, dd, dn, d_err, stream);
        if (e == cudaSuccess && leaf) e = cudaMemcpyAsync(leaf, dl, n * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess && inside) e = cudaMemcpyAsync(inside, di, n * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess && dist) e = cudaMemcpyAsync(dist, dd, n * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess && normal) e = cudaMemcpyAsync(normal, dn, (size_t)n * 12, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        cudaFree(buf);
        if (e != cudaSuccess) return cuda_fail(e, "query");
        return sync();
    }

    int set_launch(int blk, int ctas) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        const int bi = block_index(blk);
        if (bi < 0) return fail(VISG_ERR_INVALID_ARG, "block must be 128, 256, 512 or 1024");
        if (ctas < 0 || (ctas > 0 && ctas > step_max_ctas_per_sm(variant(blk), blk, win_cap[bi])))
            return fail(VISG_ERR_INVALID_ARG, "ctas_per_sm out of range for this block size");
        if (int r = sync()) return r;
        if (blk != block || ctas * sm_count != grid || reserve != 0) {
            block = blk;
            grid = ctas * sm_count;
            reserve = 0;
            destroy_graphs();
        }
        return VISG_OK;
    }

    int set_reserve(int sms) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (sms < 0 || sms >= sm_count) return fail(VISG_ERR_INVALID_ARG, "reserve out of range");
        if (int r = sync()) return r;
        if (sms != reserve) {
            reserve = sms;
            destroy_graphs();
        }
        return VISG_OK;
    }

    // time every launch shape on this engine's data; keep the fastest; restore the state
    int autotune(int* out_block, int* out_ctas) {
        if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
        if (int r = sync()) return r;
        float4 *bs = nullptr, *bn = nullptr;
        CU(cudaMalloc((void**)&bs, 4 * (size_t)N * sizeof(float4)));
        cudaError_t e = cudaMalloc((void**)&bn, (size_t)N * sizeof(float4));
        if (e != cudaSuccess) {
            cudaFree(bs);
            return cuda_fail(e, "autotune backup");
        }
        const int cur0 = cur;
        e = cudaMemcpyAsync(bs, d_state[cur], 2 * (size_t)N * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(bs + 2 * N, d_state[cur ^ 1], 2 * (size_t)N * sizeof(float4), cudaMemcpyDeviceToDevice,
                                stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(bn, d_normal, (size_t)N * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
        // every candidate starts from the same state, so all are timed on the same contacts
        auto restore = [&]() {
            cur = cur0;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_state[cur], bs, 2 * (size_t)N * sizeof(float4), cudaMemcpyDeviceToDevice,
                                    stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_state[cur ^ 1], bs + 2 * N, 2 * (size_t)N * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_normal, bn, (size_t)N * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
            // the query caches refer to the timed steps' answers
            if (e == cudaSuccess) e = launch_clear_margin(d_state[cur], 0, N, stream);
        };
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 1e30f;
        int best_block = block, best_grid = grid, best_ctas = 0, best_split = split, best_stage = stage;
        const int split0 = split, stage0 = stage;
        const int n_split = (p.collide && any_body) ? 2 : 1;
        for (int sv = 0; sv < 2 * n_split * kNumBlocks && e == cudaSuccess; ++sv) {
            stage = sv / (kNumBlocks * n_split);
            split = (sv / kNumBlocks) % n_split;
            const int bi = sv % kNumBlocks;
            const int blk = kBlocks[bi];
            if (stage && win_cap[bi] == 0) continue;
            const int occ = step_max_ctas_per_sm(variant(blk), blk, win_cap[bi]);
            std::vector<int> ctas;
            for (int c = 1; c <= occ; c *= 2) ctas.push_back(c);
            if (occ > 0 && ctas.back() != occ) ctas.push_back(occ);
            ctas.push_back(0);  // one tile per CTA
            for (int c : ctas) {
                const int gr = c == 0 ? 0 : c * sm_count;
                auto run = [&](int k) {
                    for (int s = 0; s < k && e == cudaSuccess; ++s) {
                        e = launch_step(args(cur, blk), variant(blk), blk, gr, stream);
                        cur ^= 1;
                    }
                };
                restore();
                run(1);
                cudaEventRecord(e0, stream);
                run(6);
                cudaEventRecord(e1, stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (e == cudaSuccess && ms < best) {
                    best = ms;
                    best_block = blk;
                    best_grid = gr;
                    best_ctas = c;
                    best_split = split;
                    best_stage = stage;
                }
            }
        }
        split = split0;
        stage = stage0;
        restore();
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e == cudaSuccess &&
            (best_block != block || best_grid != grid || best_split != split || best_stage != stage || reserve != 0)) {
            block = best_block;
            grid = best_grid;
            split = best_split;
            stage = best_stage;
            reserve = 0;
            destroy_graphs();
        }
        // with two overlapping chains of persistent kernels and the collision split out,
        // time whole steps, replayed from the step graphs as they run (the chains
        // overlap only there), with SMs left free for the other group's collision pass
        if (e == cudaSuccess && groups() == 2 && grid > 0 && (variant(block) & SV_SPLIT) && p.use_graph) {
            float best_r = 1e30f;
            int best_res = 0;
            for (int res : {0, 8, 16, 24, 32}) {
                if (res >= sm_count / 2 || e != cudaSuccess) break;
                reserve = res;
                destroy_graphs();
                restore();
                if (step(chunk_steps) != VISG_OK) e = cudaErrorUnknown;  // captures this shape's graph
                if (e == cudaSuccess) e = cudaEventRecord(e0, stream);
                if (e == cudaSuccess && step(2 * chunk_steps) != VISG_OK) e = cudaErrorUnknown;
                if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (e == cudaSuccess && ms < best_r) {
                    best_r = ms;
                    best_res = res;
                }
            }
            reserve = best_res;
            restore();
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
            destroy_graphs();
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(bs);
        cudaFree(bn);
        if (e != cudaSuccess) return cuda_fail(e, "autotune");
        if (out_block) *out_block = block;
        if (out_ctas) *out_ctas = best_ctas;
        return sync();
    }

    int forward(int nsteps, int ckpt);
    int backward(const float* dL_dx, const float* dL_dxo, float* dL_dk, float* dL_dscalar);
    int forward_contacts(int64_t* counts, int n);
    cudaError_t step64(int c, unsigned* contacts = nullptr);
    cudaError_t save64(int c, double* dst);
    cudaError_t load64(const double* src);
};

struct VisgSim {
    Engine eng;
};
struct VisgBatch {
    Engine eng;
};

#include "visg_adjoint_host.inl"

// =====================================================================================
// a named range around each public call, for profilers (NVTX)
struct ApiRange {
    explicit ApiRange(const char* name) { nvtxRangePushA(name); }
    ~ApiRange() { nvtxRangePop(); }
    ApiRange(const ApiRange&) = delete;
    ApiRange& operator=(const ApiRange&) = delete;
};

extern "C" {

void visg_default_params(VisgParams* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->dt = 1.0f / 40.0f;
    p->mass = 0.3f;
    p->gravity[0] = 0.0f;
    p->gravity[1] = -0.00981f;
    p->gravity[2] = 0.0f;
    p->force_damping = -0.02f;
    p->spring_damping = -0.5f;
    p->verlet_damping = 1.0f;
    p->thickness = 0.003f;
    p->box_depth = 0.01f;
    p->n_lists = 2;
    p->list_k[0] = 100.0f;
    p->list_k[1] = 2.0f;
    p->list_k[2] = 2.0f;
    p->list_k[3] = 2.0f;
    p->collide = 1;
    p->check_every = 0;
    p->max_displacement = 1.0f;
    p->use_graph = 1;
    p->split_collision = 1;
    p->stage_neighbours = 0;
    p->collision_margin = 1;
    p->overlap_groups = 0;
}

const char* visg_version(void) { return "visg-gb300 1.0 (sm_103a)"; }
const char* visg_last_error(void) { return g_err.c_str(); }

static int ensure_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(VISG_ERR_NO_DEVICE, "no CUDA device visible");
    return VISG_OK;
}

int visg_create(const VisgParams* params, const float* cloth_xyz, int32_t n_vertices, const uint32_t* const* csr_row,
                const VisgSpring* const* csr, const float* const* list_k, const float* body_xyz,
                const float* body_normals, int32_t n_body_vertices, const uint32_t* tris, int32_t n_tris,
                VisgSim** out) {
    ApiRange range_("visg_create");
    if (!out) return fail(VISG_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (int r = validate_params(params)) return r;
    if (int r = ensure_device()) return r;
    auto* s = new VisgSim();
    s->eng.p = *params;
    int r = s->eng.add(cloth_xyz, n_vertices, csr_row, csr, list_k, nullptr, 0, body_xyz, body_normals,
                       n_body_vertices, tris, n_tris, nullptr);
    if (r == VISG_OK) r = s->eng.finalize();
    if (r != VISG_OK) {
        std::string m = g_err;
        delete s;
        g_err = m;
        return r;
    }
    *out = s;
    return VISG_OK;
}

int visg_destroy(VisgSim* sim) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    delete sim;
    return VISG_OK;
}

int visg_set_stream(VisgSim* sim, void* stream) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    sim->eng.stream = (cudaStream_t)stream;
    return VISG_OK;
}

int visg_step(VisgSim* sim, int32_t nsteps) {
    ApiRange range_("visg_step");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.step(nsteps);
}

int visg_update_body(VisgSim* sim, const float* xyz, const float* nrm) {
    ApiRange range_("visg_update_body");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.update_body(0, xyz, nrm, cudaMemcpyHostToDevice);
}

int visg_update_body_device(VisgSim* sim, const float* xyz, const float* nrm) {
    ApiRange range_("visg_update_body_device");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.update_body(0, xyz, nrm, cudaMemcpyDeviceToDevice);
}

int visg_set_vertex(VisgSim* sim, uint32_t idx, const float xyz[3]) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.set_vertex(0, idx, xyz);
}

int visg_set_vertices(VisgSim* sim, const uint32_t* idx, const float* xyz, int32_t n) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.set_vertices(idx, xyz, n);
}

int visg_set_pinned(VisgSim* sim, const uint32_t* idx, int32_t n) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.set_pinned(idx, n);
}

int visg_get_positions(VisgSim* sim, float* out, int32_t on_device) {
    ApiRange range_("visg_get_positions");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.get_positions(0, out, on_device);
}

int visg_read_positions_async(VisgSim* sim, float* out) {
    ApiRange range_("visg_read_positions_async");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.read_positions_async(out);
}

int visg_wait_positions(VisgSim* sim) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.wait_positions();
}

int visg_set_faces(VisgSim* sim, const uint32_t* faces, int32_t n_faces) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.set_faces(0, faces, n_faces);
}

int visg_render(VisgSim* sim, float* pos4, float* vertex_normals, float* face_normals, int32_t on_device,
                int32_t normals_of_previous) {
    ApiRange range_("visg_render");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.render(pos4, vertex_normals, face_normals, nullptr, nullptr, on_device, normals_of_previous);
}

int visg_render_shaded(VisgSim* sim, float* pos4, float* vertex_normals, float* colors, const float object_rgb[3],
                       int32_t on_device, int32_t normals_of_previous) {
    ApiRange range_("visg_render_shaded");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.render(pos4, vertex_normals, nullptr, colors, object_rgb, on_device, normals_of_previous);
}

int visg_get_state(VisgSim* sim, float* x, float* xo, float* n) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.get_state(-1, x, xo, n);
}

int visg_set_state(VisgSim* sim, const float* x, const float* xo, const float* n) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.set_state(-1, x, xo, n);
}

int visg_sync(VisgSim* sim) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.sync();
}

int visg_count_contacts(VisgSim* sim, int64_t* n) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.count_contacts(n);
}

int visg_batch_count_contacts(VisgBatch* b, int64_t* n) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.count_contacts(n);
}

int visg_get_info(VisgSim* sim, int32_t* nv, int32_t* ne, int32_t* nt, int32_t* nl) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    Engine& e = sim->eng;
    if (nv) *nv = (int32_t)e.N;
    if (ne) *ne = (int32_t)e.E;
    if (nt) *nt = e.gin[0].nt;
    if (nl) {
        *nl = 0;
        if (e.gin[0].nt > 0) {
            if (int r = e.sync()) return r;
            BvhRoot rt;
            cudaError_t ce = cudaMemcpy(&rt, e.bvh[0].root, sizeof rt, cudaMemcpyDeviceToHost);
            if (ce != cudaSuccess) return cuda_fail(ce, "info");
            *nl = rt.n_leaves;
        }
    }
    return VISG_OK;
}

int visg_export_lbvh(VisgSim* sim, uint32_t* tri_codes, float* tri_boxes, uint32_t* sorted_codes, int32_t* sorted_tris,
                     int32_t* child_a, int32_t* child_b, int32_t* parent_internal, int32_t* parent_leaf,
                     float* internal_boxes, float* leaf_boxes, float* root_box) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.export_lbvh(0, tri_codes, tri_boxes, sorted_codes, sorted_tris, child_a, child_b, parent_internal,
                                parent_leaf, internal_boxes, leaf_boxes, root_box);
}

int visg_query_points(VisgSim* sim, const float* pts, int32_t n, int32_t* leaf, int32_t* inside, float* dist,
                      float* normal) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.query(0, pts, n, leaf, inside, dist, normal);
}

int visg_forward(VisgSim* sim, int32_t nsteps, int32_t ckpt) {
    ApiRange range_("visg_forward");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.forward(nsteps, ckpt);
}

int visg_forward_contacts(VisgSim* sim, int64_t* counts, int32_t n) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.forward_contacts(counts, n);
}

int visg_backward(VisgSim* sim, const float* dL_dx, const float* dL_dxo, float* dL_dk, float* dL_dscalar) {
    ApiRange range_("visg_backward");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.backward(dL_dx, dL_dxo, dL_dk, dL_dscalar);
}

// ---------------------------------------------------------------------------------------
int visg_batch_create(const VisgParams* params, VisgBatch** out) {
    if (!out) return fail(VISG_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (int r = validate_params(params)) return r;
    if (int r = ensure_device()) return r;
    auto* b = new VisgBatch();
    b->eng.p = *params;
    *out = b;
    return VISG_OK;
}

int visg_batch_add(VisgBatch* b, const float* cloth_xyz, int32_t n_vertices, const uint32_t* const* csr_row,
                   const VisgSpring* const* csr, const float* const* list_k, const uint32_t* pinned, int32_t n_pinned,
                   const float* body_xyz, const float* body_normals, int32_t n_body_vertices, const uint32_t* tris,
                   int32_t n_tris, int32_t* garment) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    if (n_pinned < 0 || (n_pinned > 0 && !pinned)) return fail(VISG_ERR_INVALID_ARG, "bad pin list");
    return b->eng.add(cloth_xyz, n_vertices, csr_row, csr, list_k, pinned, n_pinned, body_xyz, body_normals,
                      n_body_vertices, tris, n_tris, garment);
}

int visg_batch_finalize(VisgBatch* b) {
    ApiRange range_("visg_batch_finalize");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.finalize();
}

int visg_batch_set_stream(VisgBatch* b, void* stream) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    b->eng.stream = (cudaStream_t)stream;
    return VISG_OK;
}

int visg_batch_step(VisgBatch* b, int32_t nsteps) {
    ApiRange range_("visg_batch_step");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.step(nsteps);
}

int visg_batch_get_positions(VisgBatch* b, int32_t garment, float* out, int32_t on_device) {
    ApiRange range_("visg_batch_get_positions");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.get_positions(garment, out, on_device);
}

int visg_batch_get_state(VisgBatch* b, int32_t garment, float* x, float* x_old, float* normal) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.get_state(garment, x, x_old, normal);
}

int visg_batch_set_state(VisgBatch* b, int32_t garment, const float* x, const float* x_old, const float* normal) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.set_state(garment, x, x_old, normal);
}

int visg_batch_read_positions_async(VisgBatch* b, float* out) {
    ApiRange range_("visg_batch_read_positions_async");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.read_positions_async(out);
}

int visg_batch_wait_positions(VisgBatch* b) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.wait_positions();
}

int visg_batch_set_faces(VisgBatch* b, int32_t garment, const uint32_t* faces, int32_t n_faces) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.set_faces(garment, faces, n_faces);
}

int visg_batch_render(VisgBatch* b, float* pos4, float* vertex_normals, float* face_normals, int32_t on_device,
                      int32_t normals_of_previous) {
    ApiRange range_("visg_batch_render");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.render(pos4, vertex_normals, face_normals, nullptr, nullptr, on_device, normals_of_previous);
}

int visg_batch_render_shaded(VisgBatch* b, float* pos4, float* vertex_normals, float* colors,
                             const float object_rgb[3], int32_t on_device, int32_t normals_of_previous) {
    ApiRange range_("visg_batch_render_shaded");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.render(pos4, vertex_normals, nullptr, colors, object_rgb, on_device, normals_of_previous);
}

int visg_batch_set_vertex(VisgBatch* b, int32_t garment, uint32_t idx, const float xyz[3]) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.set_vertex(garment, idx, xyz);
}

int visg_batch_set_vertices(VisgBatch* b, const uint32_t* idx, const float* xyz, int32_t n) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.set_vertices(idx, xyz, n);
}

int visg_batch_update_body(VisgBatch* b, int32_t garment, const float* xyz, const float* nrm) {
    ApiRange range_("visg_batch_update_body");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.update_body(garment, xyz, nrm, cudaMemcpyHostToDevice);
}

int visg_batch_time_kernels(VisgBatch* b, int32_t nsteps, float* ms_step_kernel, float* ms_collide_kernel) {
    ApiRange range_("visg_batch_time_kernels");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.time_kernels(nsteps, ms_step_kernel, ms_collide_kernel);
}

int visg_selftest_bounded_waits(int32_t* gave_up) {
    ApiRange range_("visg_selftest_bounded_waits");
    if (!gave_up) return fail(VISG_ERR_INVALID_ARG, "gave_up is NULL");
    *gave_up = 0;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return fail(VISG_ERR_NO_DEVICE, "no CUDA device");
    // [0] mbarrier wait's error word, [1] look-back's, [2] a status word nothing publishes,
    // [3] grid barrier's error word, [4] an arrival counter no other CTA increments
    int* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, 32);
    if (e != cudaSuccess) return cuda_fail(e, "self-test buffer");
    int h[4] = {0, 0, 0, 0};
    e = cudaMemset(d, 0, 32);
    if (e == cudaSuccess) e = launch_selftest_mbar_wait(d, nullptr);
    if (e == cudaSuccess) e = launch_selftest_look_back(reinterpret_cast<const uint32_t*>(d + 2), d + 1, nullptr);
    if (e == cudaSuccess) e = launch_selftest_grid_wait(reinterpret_cast<uint32_t*>(d + 4), d + 3, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    // the device must still work after the waits gave up
    if (e == cudaSuccess) e = cudaMemset(d, 0, 32);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "self-test of the bounded waits");
    *gave_up = ((h[0] & ERR_TIMEOUT) ? 1 : 0) | ((h[1] & ERR_TIMEOUT) ? 2 : 0) | ((h[3] & ERR_TIMEOUT) ? 4 : 0);
    return VISG_OK;
}

int visg_selftest_exact_math(uint64_t* checked, uint64_t* mismatches) {
    ApiRange range_("visg_selftest_exact_math");
    if (!checked || !mismatches) return fail(VISG_ERR_INVALID_ARG, "NULL output");
    *checked = *mismatches = 0;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return fail(VISG_ERR_NO_DEVICE, "no CUDA device");
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, 3 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "self-test buffer");
    unsigned long long h[3] = {0, 0, 0};
    e = cudaMemset(d, 0, sizeof h);
    if (e == cudaSuccess) e = launch_selftest_exact_math(d, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "self-test of the packed square root and reciprocal");
    *checked = h[0];
    *mismatches = h[1] + h[2];
    return VISG_OK;
}

int visg_batch_autotune(VisgBatch* b, int32_t* block, int32_t* ctas) {
    ApiRange range_("visg_batch_autotune");
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.autotune(block, ctas);
}

int visg_batch_set_launch(VisgBatch* b, int32_t block, int32_t ctas) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.set_launch(block, ctas);
}

static int launch_info(const Engine& e, int32_t* block, int32_t* ctas, int32_t* split, int32_t* stage,
                       int32_t* kernels) {
    const int v = e.variant(e.block);
    if (block) *block = e.block;
    if (ctas) *ctas = e.sm_count > 0 ? e.grid / e.sm_count : 0;
    if (split) *split = (v & SV_SPLIT) ? 1 : 0;
    if (stage) *stage = (v & SV_STAGED) ? 1 : 0;
    if (kernels) *kernels = ((v & SV_SPLIT) ? 2 : 1) * e.groups();
    return VISG_OK;
}

int visg_batch_launch_info(VisgBatch* b, int32_t* block, int32_t* ctas, int32_t* split, int32_t* stage,
                           int32_t* kernels) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return launch_info(b->eng, block, ctas, split, stage, kernels);
}

int visg_batch_set_reserve(VisgBatch* b, int32_t sms) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    return b->eng.set_reserve(sms);
}

int visg_batch_get_reserve(VisgBatch* b, int32_t* sms) {
    if (!b || !sms) return fail(VISG_ERR_INVALID_ARG, "batch or sms is NULL");
    *sms = b->eng.step_grid() != b->eng.grid ? b->eng.reserve : 0;
    return VISG_OK;
}

int visg_autotune(VisgSim* sim, int32_t* block, int32_t* ctas) {
    ApiRange range_("visg_autotune");
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return sim->eng.autotune(block, ctas);
}

int visg_launch_info(VisgSim* sim, int32_t* block, int32_t* ctas, int32_t* split, int32_t* stage, int32_t* kernels) {
    if (!sim) return fail(VISG_ERR_INVALID_ARG, "sim is NULL");
    return launch_info(sim->eng, block, ctas, split, stage, kernels);
}

int visg_batch_info(VisgBatch* b, int32_t* ng, int64_t* nv, int64_t* ne, int64_t* nt) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    Engine& e = b->eng;
    if (ng) *ng = (int32_t)e.gin.size();
    if (nv) *nv = e.N;
    if (ne) {
        int64_t s = 0;
        for (auto& g : e.gin)
            for (auto& r : g.rows) s += r.back();
        *ne = s;
    }
    if (nt) {
        int64_t s = 0;
        for (auto& g : e.gin) s += g.nt;
        *nt = s;
    }
    return VISG_OK;
}

int visg_batch_sync(VisgBatch* b) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    if (!b->eng.finalized) return VISG_OK;
    return b->eng.sync();
}

int visg_batch_destroy(VisgBatch* b) {
    if (!b) return fail(VISG_ERR_INVALID_ARG, "batch is NULL");
    delete b;
    return VISG_OK;
}

}  // extern "C"
