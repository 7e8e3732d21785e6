// visg_lbvh_static.cu — the body LBVH build without any device allocation.
//
// Some callers of this library cannot call cudaMalloc: a host application whose
// own allocator owns the whole device (a pooling allocator or an arena sized at
// start-up), code that runs where allocation is forbidden or would synchronise the
// device at a bad moment, or a plugin that must not change the process's memory
// footprint after initialisation.  visg_lbvh_build_noalloc serves them: the caller
// passes the body (device pointers) and the output arrays, and every temporary the
// build needs (boxes, Morton codes, radix-sort buffers, look-back status words,
// chunk summaries) lives in one file-scope __device__ array, so the call itself
// allocates nothing.
//
// Costs and limits:
//   * the array (VISG_NOALLOC_SCRATCH_BYTES) is reserved on every GPU that loads
//     this library and held until the process exits;
//   * bodies are limited to VISG_NOALLOC_MAX_VERTICES vertices and
//     VISG_NOALLOC_MAX_TRIS triangles; larger inputs are rejected;
//   * all calls share the array and it keeps the last call's contents: the build
//     clears what must start at zero itself, and two calls whose GPU work overlaps
//     (different streams, or different host threads) race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "visg_internal.cuh"

using namespace visg;

namespace {

constexpr size_t kScratchBytes = VISG_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_lbvh_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};  // device address of g_lbvh_scratch, per device

int bad(int code) { return code; }

// The array's name in host code is a host-side stand-in, not a device address:
// look the address up once per device, with that device current.
int scratch_address(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return bad(VISG_ERR_NO_DEVICE);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
        if (e != cudaSuccess || !p) return bad(VISG_ERR_CUDA);
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return VISG_OK;
}

// Reference layout of the links (BRTreeNode, cudaBRT.h:34-115): the root is
// internal node 0; an internal node that is child A takes the index of its last
// leaf, child B of its first.  Pass 1 gives every internal node its index.
// Both passes run only on a build that reported no error, and check every index
// they read from the tree before using it: a build whose bounded wait gave up can
// leave the shared array with another call's nodes, and nothing read from there may
// send a store outside the caller's arrays.  A bad index sets ERR_INDEX instead.
__device__ __forceinline__ bool tree_ok(const BvhRoot* root, const int* err, int n_tris, int& n) {
    n = root->n_leaves;
    return *err == 0 && n >= 2 && n <= n_tris;
}

__global__ void k_karras_index(const Node* __restrict__ nodes, const int2* __restrict__ range,
                               const BvhRoot* __restrict__ root, int* __restrict__ kidx, int n_tris, int* err) {
    int n;
    if (!tree_ok(root, err, n_tris, n)) return;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n - 1) return;
    if (g == root->root) kidx[g] = 0;
    const int la = __float_as_int(nodes[g].a_lo.w), lb = __float_as_int(nodes[g].b_lo.w);
    if (la >= n - 1 || lb >= n - 1) {
        atomicOr(err, ERR_INDEX);
        return;
    }
    if (la >= 0) kidx[la] = range[la].y;
    if (lb >= 0) kidx[lb] = range[lb].x;
}

// Pass 2: child links in the reference encoding (+(i+1) internal, -(i+1) leaf).
__global__ void k_karras_links(const Node* __restrict__ nodes, const BvhRoot* __restrict__ root,
                               const int* __restrict__ kidx, int32_t* __restrict__ child_a,
                               int32_t* __restrict__ child_b, int n_tris, int* err) {
    int n;
    if (!tree_ok(root, err, n_tris, n)) return;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n - 1) return;
    const int k = kidx[g];
    const int la = __float_as_int(nodes[g].a_lo.w), lb = __float_as_int(nodes[g].b_lo.w);
    if (k < 0 || k >= n - 1 || la >= n - 1 || lb >= n - 1) {
        atomicOr(err, ERR_INDEX);
        return;
    }
    child_a[k] = la < 0 ? -(~la) - 1 : kidx[la] + 1;
    child_b[k] = lb < 0 ? -(~lb) - 1 : kidx[lb] + 1;
}

// Leaf count to the caller; -1 if a bounded wait of the build gave up or an index
// was out of range (a triangle's vertex index, or one read from the tree).
__global__ void k_report(const BvhRoot* __restrict__ root, const int* __restrict__ err, int32_t* n_leaves) {
    *n_leaves = *err ? -1 : root->n_leaves;
}

}  // namespace

extern "C" int visg_lbvh_build_noalloc(const float* d_xyz, const float* d_normals, int32_t n_vertices,
                                       const uint32_t* d_tris, int32_t n_tris, float thickness, float box_depth,
                                       uint32_t* d_sorted_codes, int32_t* d_sorted_tris, int32_t* d_child_a,
                                       int32_t* d_child_b, int32_t* d_n_leaves, void* cuda_stream) {
    if (!d_xyz || !d_tris || !d_sorted_codes || !d_sorted_tris || !d_n_leaves || (n_tris > 1 && (!d_child_a || !d_child_b)))
        return bad(VISG_ERR_INVALID_ARG);  // a NULL pointer
    if (n_vertices < 1 || n_tris < 1) return bad(VISG_ERR_INVALID_ARG);  // empty body
    // larger than the static scratch holds: such bodies go through visg_create / visg_update_body
    if (n_vertices > VISG_NOALLOC_MAX_VERTICES || n_tris > VISG_NOALLOC_MAX_TRIS) return bad(VISG_ERR_INVALID_ARG);
    void* base = nullptr;
    if (int r = scratch_address(&base)) return r;
    cudaStream_t s = (cudaStream_t)cuda_stream;

    // carve the build's buffers out of the static array (the same plan the
    // allocating path uses), then point inputs and outputs at the caller's arrays
    BvhBuffers b;
    Arena plan;
    b.plan(plan, n_vertices, n_tris, d_normals != nullptr);
    int* d_err = nullptr;
    int* kidx = nullptr;
    plan.want(&d_err, 4);
    plan.want(&kidx, (size_t)n_tris + 1);
    size_t used = 0;
    for (auto& pl : plan.plan) used += pl.second;
    if (used > kScratchBytes) return bad(VISG_ERR_UNSUPPORTED);  // cannot happen within the size limits
    char* p = (char*)base;
    for (auto& pl : plan.plan) {
        *pl.first = p;
        p += pl.second;
    }
    b.xyz_in = const_cast<float*>(d_xyz);
    b.nrm_in = const_cast<float*>(d_normals);
    b.tris = const_cast<uint32_t*>(d_tris);
    b.ucode = d_sorted_codes;
    b.utri = reinterpret_cast<uint32_t*>(d_sorted_tris);

    // what must start at zero: the error word and the build's grid-barrier counters
    // (the array holds the last call's data, laid out for its sizes); the build
    // clears its histograms, look-back status words and tile counters itself
    cudaError_t e = cudaMemsetAsync(d_err, 0, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.sync, 0, 2 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = lbvh_build(b, thickness, box_depth, d_err, s);
    if (e == cudaSuccess && n_tris > 1) {
        const unsigned grid = (unsigned)((n_tris + 255) / 256);
        k_karras_index<<<grid, 256, 0, s>>>(b.nodes, b.range, b.root, kidx, n_tris, d_err);
        k_karras_links<<<grid, 256, 0, s>>>(b.nodes, b.root, kidx, d_child_a, d_child_b, n_tris, d_err);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_report<<<1, 1, 0, s>>>(b.root, d_err, d_n_leaves);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? VISG_OK : bad(VISG_ERR_CUDA);
}
