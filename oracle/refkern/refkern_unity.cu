// Unity translation unit for "refkern": the VISGSim reference's own hot-path CUDA
// kernels compiled, unmodified, into one sm_103a cubin that the host harness
// (refharness.cpp) loads through the CUDA driver API.
//
//   verlet.cu        -> verlet, update_vbo_pos, compute_face_normal, compute_vbo_normal
//   bvh/cudaBRT.cu   -> processInternalNode, calculateBoudingBox, D_BVH::intersect
//   bvh/primitive.cu -> expanded boxes, point/plane test
//   bvh_fixed.cu     -> a build-time copy of bvh/bvh.cu with its one syntax error
//                       (bvh.cu:33, "float x = p.x, float y = ...") corrected;
//                       provides compute_morton_bbox and init_nodes.
//
// Built only where the reference tree is present, by oracle/build.py, with
// --fmad=false so each source-level float operation is one IEEE operation.
// Test infrastructure: nothing in the shipped library links or loads it.
#include <cfloat>
// bvh.cu includes thrust after primitive.h has defined a `uint` macro that breaks
// the CCCL headers; parsing them first keeps their include guards ahead of it.
#include <thrust/sort.h>
#include <thrust/execution_policy.h>
#include "verlet.cu"
#include "bvh/cudaBRT.cu"
#include "bvh/primitive.cu"
#include "bvh_fixed.cu"
