/*
 * visg_sim.h — C ABI of the GB300-native VISGSim cloth step.
 *
 * Drop-in boundary for the reference's `Simulator` class (src/simulator.h:9-59):
 * plain C types, pointers and sizes only; every call returns an int status
 * (VISG_OK = 0, negative on error) and never throws.  One handle owns all of its
 * device memory; calls on one handle are not thread-safe; calls on different
 * handles are independent.  Work is issued on the handle's CUDA stream
 * (visg_set_stream; the legacy default stream unless set) and is asynchronous
 * unless the function says it synchronises.
 *
 * Physics follows src/verlet.cu:24-161 (fused Verlet step, damped CSR springs,
 * inelastic force projection and first-hit BVH position projection) and the LBVH
 * of src/bvh/{bvh.cu,cudaBRT.cu,primitive.cu,bbox.h}.  Where the reference is
 * undefined or buggy the behaviour chosen here is stated next to the call.
 */
#ifndef VISG_SIM_H
#define VISG_SIM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define VISG_OK               0
#define VISG_ERR_INVALID_ARG (-1) /* bad size, null pointer, index out of range      */
#define VISG_ERR_CUDA        (-2) /* a CUDA runtime call failed; see visg_last_error */
#define VISG_ERR_OOM         (-3) /* device allocation failed                        */
#define VISG_ERR_NO_DEVICE   (-4) /* no CUDA device visible                          */
#define VISG_ERR_DIVERGED    (-5) /* NaN/Inf or displacement above the limit seen    */
#define VISG_ERR_TIMEOUT     (-6) /* a bounded device-side wait gave up              */
#define VISG_ERR_STATE       (-7) /* call not valid in the handle's current state    */
#define VISG_ERR_UNSUPPORTED (-8) /* input the chosen path cannot handle             */

#define VISG_MAX_LISTS 4

/* One directed CSR spring entry.  Same layout as the reference's s_spring
 * (src/spring.h:8-12): `end` is the other vertex, `rest` the rest length. */
typedef struct VisgSpring {
    int32_t end;
    float rest;
} VisgSpring;

/* Physics and pipeline parameters.  visg_default_params() fills the reference's
 * constants (src/verlet.cu:12-21,62; src/simulation.cu:132; src/bvh/primitive.cu:21). */
typedef struct VisgParams {
    float dt;              /* time step                              (verlet.cu:17, 1/40)      */
    float mass;            /* per-vertex mass                        (verlet.cu:16, 0.3)       */
    float gravity[3];      /* acceleration                           (verlet.cu:19-21)         */
    float force_damping;   /* F += force_damping * v                 (verlet.cu:15, -0.02)     */
    float spring_damping;  /* kd of every spring                     (verlet.cu:62, -0.5)      */
    float verlet_damping;  /* gamma: x' = x + gamma*(x - x_old) + a dt^2.  Exactly 1.0 selects
                              the reference expression 2x - x_old + a dt^2 (verlet.cu:155).      */
    float thickness;       /* body vertices pushed along their normal once per body upload
                              (Mesh::vertex_extend, Mesh.cpp:101-117; simulation.cu:132, 0.003) */
    float box_depth;       /* expanded triangle box depth            (primitive.cu:21, 0.01)   */
    int32_t n_lists;       /* number of spring lists, 1..VISG_MAX_LISTS (reference: 2)         */
    float list_k[VISG_MAX_LISTS]; /* stiffness of each list          (verlet.cu:13-14, 100, 2) */
    int32_t collide;       /* 1: body collision on (reference), 0: off                          */
    int32_t check_every;   /* every K steps check for NaN/Inf and |dx| > max_displacement; 0=off */
    float max_displacement;/* limit for the divergence check (metres per step)                  */
    int32_t use_graph;     /* 1: replay multi-step loops as CUDA graphs (default), 0: launches  */
    int32_t split_collision; /* 1: collision in its own kernel over the vertices inside a body's
                                box (default), 0: fused into the step kernel; same results.
                                visg_autotune / visg_batch_autotune may change it.             */
    int32_t stage_neighbours; /* 1: each tile's block of spring entries is staged in shared
                                memory by TMA bulk copies, 0: read through the L1 (default);
                                same results.  visg_autotune / visg_batch_autotune may change it. */
    int32_t collision_margin; /* 1: each vertex caches its last first-hit query's answer with
                                a margin (how far it may move before any box the query
                                tested could answer differently) and reuses the answer
                                while it stays within it, redoing only the plane test
                                (default); 0: query every step.  Same results;
                                update_body clears the caches.                           */
    int32_t overlap_groups;  /* batches: 0 (default) steps the garments as two groups of about
                                equal vertex count, each its own chain of kernels on its own
                                stream inside the step graphs, so one group's collision pass
                                and kernel boundaries overlap the other's step; 1: one chain.
                                Same results.                                             */
} VisgParams;

void visg_default_params(VisgParams* p);

/* Library / device information.  Returns a static string; never NULL. */
const char* visg_version(void);
/* Message of the last failing call on this thread (any handle); never NULL. */
const char* visg_last_error(void);

/* ======================================================================== */
/* Plain form: one garment, one body.                                         */
/* ======================================================================== */
typedef struct VisgSim VisgSim;

/* Replaces Simulator(Mesh& cloth, Mesh& body) (src/simulation.cu:47-100,102-125,127-138).
 *   cloth_xyz   n_vertices*3 floats; initial x and x_old (zero velocity, simulation.cu:84-85)
 *   csr_row[l]  n_vertices+1 row offsets of spring list l (CSR_R_*, simulator.h:45-46)
 *   csr[l]      csr_row[l][n_vertices] entries of list l (CSR_C_*), entries of one row in
 *               the order the forces are summed
 *   list_k      NULL, or per list NULL / one stiffness per entry of that list (overrides
 *               params->list_k[l] entry by entry; needed for per-spring gradients)
 *   body_xyz    n_body_vertices*3 floats, body_normals NULL or n_body_vertices*3 floats;
 *               with normals the vertices are pushed by params->thickness along them
 *   tris        n_tris*3 vertex indices.  n_tris == 0 disables collision.
 * The LBVH is built before the call returns (asynchronously on the stream). */
int visg_create(const VisgParams* params,
                const float* cloth_xyz, int32_t n_vertices,
                const uint32_t* const* csr_row, const VisgSpring* const* csr,
                const float* const* list_k,
                const float* body_xyz, const float* body_normals, int32_t n_body_vertices,
                const uint32_t* tris, int32_t n_tris,
                VisgSim** out);

/* Frees everything (~Simulator, simulation.cu:28-45). Synchronises the stream. */
int visg_destroy(VisgSim* sim);

/* Launch subsequent work on `cuda_stream` (a cudaStream_t; NULL = legacy default). */
int visg_set_stream(VisgSim* sim, void* cuda_stream);

/* Replaces Simulator::simulate (simulation.cu:141-150) without the GL update:
 * `nsteps` fused steps, ping-ponging the state buffers (swap_buffer, :243-251). */
int visg_step(VisgSim* sim, int32_t nsteps);

/* New (the reference has no moving body): upload new body vertex positions (and
 * normals, for the thickness push) and rebuild the LBVH on the device:
 * expanded boxes -> root box -> Morton codes -> sort (the codes that changed since
 * the last build merged into its order, or a radix sort) -> de-duplication ->
 * radix-tree build and refit (bvh.cu:154-297, cudaBRT.cu:120-206). */
int visg_update_body(VisgSim* sim, const float* body_xyz, const float* body_normals);

/* Same with the vertices already in device memory (n_body_vertices*3 floats), read
 * by the rebuild in stream order: the arrays must stay valid until the library's
 * stream has run it. */
int visg_update_body_device(VisgSim* sim, const float* d_body_xyz, const float* d_body_normals);

/* Replaces Simulator::update_vertex (simulation.cu:253-257): sets x and x_old of
 * one vertex (its velocity becomes zero). */
int visg_set_vertex(VisgSim* sim, uint32_t idx, const float xyz[3]);

/* update_vertex for many vertices in one call: idx[k] gets x = x_old = xyz[3k..3k+2].
 * One host-to-device copy and one scatter kernel, asynchronous on the stream (the
 * host arrays are staged before the call returns).  Duplicate indices: the last wins. */
int visg_set_vertices(VisgSim* sim, const uint32_t* idx, const float* xyz, int32_t n);

/* Pinned vertices keep x and get x_old = x every step (the reference's drag via
 * update_vertex called before every step). n == 0 clears all pins. */
int visg_set_pinned(VisgSim* sim, const uint32_t* idx, int32_t n);

/* Headless replacement of cuda_update_vbo's position upload (simulation.cu:196-216):
 * writes n_vertices*3 floats of the current positions.  on_device = 1: `out` is a
 * device pointer and the copy is asynchronous; 0: host pointer (pinned or pageable),
 * synchronises and reports any device-side error (divergence, timeout). */
int visg_get_positions(VisgSim* sim, float* out, int32_t on_device);

/* The rest of cuda_update_vbo (simulation.cu:196-231), headless.  visg_set_faces gives
 * the cloth's triangles (as the Simulator constructor takes them from the Mesh,
 * simulation.cu:88-95); visg_render then writes, into caller buffers (device when
 * on_device = 1, else host; any may be NULL): pos4 = n_vertices x (x, y, z, 1)
 * (update_vbo_pos, verlet.cu:119-127), face_normals = n_faces x 3
 * (compute_face_normal, verlet.cu:91-116: normalize(cross(p1 - p0, p2 - p0))) and
 * vertex_normals = n_vertices x 3 (compute_vbo_normal, verlet.cu:163-181: the
 * normalised sum of the vertex's face normals in face order; NaN for a vertex with
 * no face, as there).  With normals_of_previous = 1 the normals are of the positions
 * the last step started from, as the reference computes them; 0 uses the current
 * positions (also the case before the first step and after visg_set_state).  Host
 * outputs synchronise and report device-side errors. */
int visg_set_faces(VisgSim* sim, const uint32_t* faces, int32_t n_faces);
int visg_render(VisgSim* sim, float* pos4, float* vertex_normals, float* face_normals, int32_t on_device,
                int32_t normals_of_previous);
/* visg_render plus, per vertex, the colour the reference's fragment shader gives it
 * (src/shaders/sh.frag:13-55, evaluated at the vertex normal instead of per fragment):
 * the order-2 spherical-harmonic irradiance polynomial with its "old town square"
 * coefficients, term by term in the shader's order, times object_rgb (its texture
 * lookup is dropped; ambient and specular are zero there).  colors: n_vertices x 3. */
int visg_render_shaded(VisgSim* sim, float* pos4, float* vertex_normals, float* colors, const float object_rgb[3],
                       int32_t on_device, int32_t normals_of_previous);

/* Pipelined read-back (no counterpart in the reference, whose cuda_update_vbo
 * copies synchronously every frame): enqueues, behind the steps issued so far, the
 * copy of all n_vertices*3 positions into host memory `out` (page-locked memory
 * lets the copy run asynchronously) and returns at once, so the steps issued next
 * run while the copy proceeds.  At most three reads may be in flight; `out` must
 * stay valid until visg_wait_positions has returned for it.  visg_wait_positions
 * waits for the oldest read in flight and reports device-side errors raised up to
 * the step it read. */
int visg_read_positions_async(VisgSim* sim, float* out);
int visg_wait_positions(VisgSim* sim);

/* Full step state (x, x_old, previous contact normal; n_vertices*3 floats each, host).
 * Any pointer may be NULL.  get synchronises. */
int visg_get_state(VisgSim* sim, float* x, float* x_old, float* normal);
int visg_set_state(VisgSim* sim, const float* x, const float* x_old, const float* normal);

/* Waits for the stream; returns the first device-side error recorded since the
 * last call (VISG_ERR_DIVERGED, VISG_ERR_TIMEOUT) or VISG_OK. */
int visg_sync(VisgSim* sim);

/* Number of vertices whose last step ended in contact (stored normal non-zero). Synchronises. */
int visg_count_contacts(VisgSim* sim, int64_t* n);

int visg_get_info(VisgSim* sim, int32_t* n_vertices, int32_t* n_entries,
                  int32_t* n_tris, int32_t* n_leaves);

/* Times the candidate launch shapes and variants of the step kernel (tile size,
 * persistent CTAs per SM, collision split into its own kernel or fused, spring
 * entries staged or not) on this simulator's own data from its current state, keeps
 * the fastest and leaves the state unchanged, as visg_batch_autotune does for a
 * batch; *block and *ctas_per_sm (may be NULL) report the choice.  For one garment
 * the fused collision usually wins: a step is then one kernel.  No counterpart in the
 * reference (it launches one fixed shape). */
int visg_autotune(VisgSim* sim, int32_t* block, int32_t* ctas_per_sm);
/* The launch shape and variant in use, as visg_batch_launch_info. */
int visg_launch_info(VisgSim* sim, int32_t* block, int32_t* ctas_per_sm, int32_t* split_collision,
                     int32_t* stage_neighbours, int32_t* kernels_per_step);

/* Inspection of the current LBVH in the reference's layout (bvh.cu:264-297,
 * cudaBRT.h:34-115).  Arrays are host memory sized for n_tris (per-triangle) or
 * n_leaves = T' (after de-duplication); any pointer may be NULL.
 *   tri_codes[T], tri_boxes[T*6] (min xyz, max xyz) — per input triangle
 *   sorted_codes[T'], sorted_tris[T']
 *   child_a/child_b/parent_internal[T'-1], parent_leaf[T'] — encoded as in
 *       BRTreeNode: +(i+1) internal, -(i+1) leaf, 0 none; root is internal 0
 *   internal_boxes[(T'-1)*6], leaf_boxes[T'*6], root_box[6] (the Morton frame)
 * Synchronises. */
int visg_export_lbvh(VisgSim* sim, uint32_t* tri_codes, float* tri_boxes,
                     uint32_t* sorted_codes, int32_t* sorted_tris,
                     int32_t* child_a, int32_t* child_b,
                     int32_t* parent_internal, int32_t* parent_leaf,
                     float* internal_boxes, float* leaf_boxes, float* root_box);

/* First-hit query of the current LBVH (D_BVH::intersect + primitive_intersect,
 * cudaBRT.cu:239-289, primitive.cu:110-125) for n host points: leaf[i] = the leaf
 * index (sorted order) or -1, inside[i] = plane test, dist[i], normal[i*3].
 * Any output may be NULL.  Synchronises. */
int visg_query_points(VisgSim* sim, const float* points, int32_t n,
                      int32_t* leaf, int32_t* inside, float* dist, float* normal);

/* ---- differentiation (hand-written adjoint) ---------------------------------
 * visg_forward runs `nsteps` steps recording a checkpoint of (x, x_old, normal)
 * every `checkpoint_every` steps; the contact set of each step is frozen as the
 * forward pass found it.  visg_backward then propagates dL/dx_final (and optional
 * dL/dx_old_final), n_vertices*3 host floats, back through those steps,
 * recomputing the steps between checkpoints, and writes
 *   dL_dk[e]     per CSR entry, lists concatenated in order (host, total entries)
 *   dL_dscalar[3] = dL/d verlet_damping, dL/d force_damping, dL/d spring_damping.
 * Requires a symmetric spring graph (every i->j entry has a j->i entry in the
 * same list); VISG_ERR_UNSUPPORTED otherwise.  Body is held static.  If a gradient
 * is not finite in float (the trajectory's sensitivity overflowed) the values are
 * written as computed and VISG_ERR_DIVERGED is returned. */
int visg_forward(VisgSim* sim, int32_t nsteps, int32_t checkpoint_every);
int visg_backward(VisgSim* sim, const float* dL_dx, const float* dL_dxold,
                  float* dL_dk, float* dL_dscalar);
/* The frozen active set of the last visg_forward, as counts: counts[s] = vertices
 * projected onto the body in forward step s, for s < n <= nsteps.  Synchronises. */
int visg_forward_contacts(VisgSim* sim, int64_t* counts, int32_t n);

/* ======================================================================== */
/* Batched form: many garments, each with its own body; every launch covers many garments
 * (two garment groups as overlapping chains of kernels per step by default).  */
/* ======================================================================== */
typedef struct VisgBatch VisgBatch;

int visg_batch_create(const VisgParams* params, VisgBatch** out);
/* Adds one garment with its body; arguments as visg_create plus pins.  Returns the
 * garment id in *garment.  Only valid before visg_batch_finalize. */
int visg_batch_add(VisgBatch* b,
                   const float* cloth_xyz, int32_t n_vertices,
                   const uint32_t* const* csr_row, const VisgSpring* const* csr,
                   const float* const* list_k,
                   const uint32_t* pinned, int32_t n_pinned,
                   const float* body_xyz, const float* body_normals, int32_t n_body_vertices,
                   const uint32_t* tris, int32_t n_tris,
                   int32_t* garment);
/* Uploads all garments, builds every body's LBVH.  After this, step/query calls. */
int visg_batch_finalize(VisgBatch* b);
int visg_batch_set_stream(VisgBatch* b, void* cuda_stream);
/* nsteps persistent launches (one per step) over all garments; with use_graph the
 * loop is replayed from a captured CUDA graph. */
int visg_batch_step(VisgBatch* b, int32_t nsteps);
/* garment = -1: all garments concatenated in id order. */
int visg_batch_get_positions(VisgBatch* b, int32_t garment, float* out, int32_t on_device);
/* visg_get_state / visg_set_state of one garment (garment = -1: all, concatenated). */
int visg_batch_get_state(VisgBatch* b, int32_t garment, float* x, float* x_old, float* normal);
int visg_batch_set_state(VisgBatch* b, int32_t garment, const float* x, const float* x_old, const float* normal);
/* visg_set_faces for one garment (local vertex indices); visg_render over all
 * garments, concatenated in id order (face normals: garment 0's faces first). */
int visg_batch_set_faces(VisgBatch* b, int32_t garment, const uint32_t* faces, int32_t n_faces);
int visg_batch_render(VisgBatch* b, float* pos4, float* vertex_normals, float* face_normals, int32_t on_device,
                      int32_t normals_of_previous);
int visg_batch_render_shaded(VisgBatch* b, float* pos4, float* vertex_normals, float* colors,
                             const float object_rgb[3], int32_t on_device, int32_t normals_of_previous);
/* visg_read_positions_async / visg_wait_positions over all garments (concatenated). */
int visg_batch_read_positions_async(VisgBatch* b, float* out);
int visg_batch_wait_positions(VisgBatch* b);
int visg_batch_set_vertex(VisgBatch* b, int32_t garment, uint32_t idx, const float xyz[3]);
/* visg_set_vertices over the whole batch: idx are global vertex indices (garments
 * concatenated in id order). */
int visg_batch_set_vertices(VisgBatch* b, const uint32_t* idx, const float* xyz, int32_t n);
int visg_batch_update_body(VisgBatch* b, int32_t garment, const float* body_xyz,
                           const float* body_normals);
/* Times the candidate launch shapes of the step kernel on this batch's own data
 * and keeps the fastest; *block and *ctas_per_sm (may be NULL) report the choice.
 * Leaves the simulation state unchanged. */
int visg_batch_autotune(VisgBatch* b, int32_t* block, int32_t* ctas_per_sm);
/* Sets the step kernel's launch shape directly (no timing): block = 128, 256, 512
 * or 1024 vertices per tile; ctas_per_sm = persistent CTAs per SM (1 .. what fits), or
 * 0 for one CTA per tile.  For reproducible timings and for callers that tune
 * offline.  No counterpart in the reference (it launches one fixed shape). */
int visg_batch_set_launch(VisgBatch* b, int32_t block, int32_t ctas_per_sm);
/* SMs the step kernel leaves free when the batch steps as two overlapping chains with
 * persistent CTAs, so that one garment group's collision pass runs beside the other
 * group's step kernel instead of after it; 0 = none (what visg_batch_set_launch
 * sets).  visg_batch_autotune chooses it by timing whole steps.  Same results.  No
 * counterpart in the reference. */
int visg_batch_set_reserve(VisgBatch* b, int32_t sms);
/* The SMs left free in the step as it runs now (0 when the launch shape or the single
 * chain makes the reserve inapplicable). */
int visg_batch_get_reserve(VisgBatch* b, int32_t* sms);
/* The launch shape and variant in use (any pointer may be NULL): block, ctas_per_sm
 * (0 = one CTA per tile), split_collision and stage_neighbours as chosen (by the
 * parameters or visg_batch_autotune), and the kernels one step launches. */
int visg_batch_launch_info(VisgBatch* b, int32_t* block, int32_t* ctas_per_sm, int32_t* split_collision,
                           int32_t* stage_neighbours, int32_t* kernels_per_step);
/* Steps the batch nsteps times as one chain of kernels (each launch covers every
 * garment), with CUDA events right around each launch of the step kernel and after
 * each collision pass on the step stream, and returns the average device time in
 * milliseconds per launch of each (ms_collide_kernel may be NULL; 0 without split
 * collision).  The steps are real steps of the simulation.  For measurement. */
int visg_batch_time_kernels(VisgBatch* b, int32_t nsteps, float* ms_step_kernel, float* ms_collide_kernel);
int visg_batch_info(VisgBatch* b, int32_t* n_garments, int64_t* n_vertices,
                    int64_t* n_entries, int64_t* n_tris);
int visg_batch_count_contacts(VisgBatch* b, int64_t* n);
int visg_batch_sync(VisgBatch* b);
int visg_batch_destroy(VisgBatch* b);

/* ======================================================================== */
/* Host-side scene helpers (no GPU needed).                                   */
/* ======================================================================== */

/* Reference spring topology from a triangle mesh (Springs::create_neigh +
 * CSR_spring, src/spring.cpp:286-353,374-391): list 0 = structure springs (unique
 * edge neighbours in face order), list 1 = bend springs (vertices opposite across
 * each shared edge).  rest = initial distance.  Call with NULL outputs to get the
 * entry counts, then again with arrays of n_vertices+1 rows and the counted entries. */
int visg_springs_from_mesh(const float* xyz, int32_t n_vertices,
                           const uint32_t* tris, int32_t n_tris,
                           uint32_t* row0, VisgSpring* ent0, int32_t* n_ent0,
                           uint32_t* row1, VisgSpring* ent1, int32_t* n_ent1);
/* visg_springs_from_mesh for a multi-piece garment (the reference's
 * SINGLE_LAYER_BOUNDARY, Springs::get_cloth_boundary_spring and
 * get_boundary_boundary_spring, spring.cpp:98-209): the vertices come in groups
 * (piece, its boundary, piece, its boundary, ...; n_groups even, sizes as
 * visg_obj_groups gives them).  Each boundary vertex is joined both ways to its
 * nearest vertex of its own piece, and the pieces' vertices behind two boundary
 * vertices that are nearest neighbours across boundaries (closer than 50 times the
 * mean boundary-to-piece distance, and apart) are joined: the seams.  These are
 * appended to the structure list after the faces' springs, in the reference's order;
 * nearest neighbours follow the rules of the reference's kd-tree (ties included). */
int visg_springs_from_mesh_sewn(const float* xyz, int32_t n_vertices, const uint32_t* tris, int32_t n_tris,
                                const int32_t* group_sizes, int32_t n_groups, uint32_t* row0, VisgSpring* ent0,
                                int32_t* n0, uint32_t* row1, VisgSpring* ent1, int32_t* n1);

/* ---- real-mesh inputs (host only, no GPU) ---------------------------------------------
 * visg_obj_load reads a Wavefront OBJ as the reference's ObjLoader + Mesh::unified do
 * (ObjLoader.cpp:14-137, Mesh.cpp:17-38), without textures and materials: "v", "vn"
 * and triangle "f" records in the "a b c" and "a/t/n b/t/n c/t/n" forms (1-based; the
 * first three corners of a face); each vertex's normal is the one named by the last
 * face corner that uses it ((0, 0, 0) for an unused vertex).  visg_obj_get copies out
 * n_vertices x 3 positions and normals and n_faces x 3 vertex indices (0-based; any
 * pointer may be NULL); visg_obj_free releases the object. */
typedef struct VisgObj VisgObj;
int visg_obj_load(const char* path, VisgObj** out, int32_t* n_vertices, int32_t* n_faces);
int visg_obj_get(const VisgObj* obj, float* xyz, float* normals, uint32_t* faces);
/* The vertex groups of a multi-piece garment: the "# object NAME" records, each sized
 * by the "# N vertices" record after it (ObjLoader.cpp:33-40), in file order: piece 0,
 * its boundary, piece 1, its boundary, ...  sizes may be NULL (count only). */
int visg_obj_groups(const VisgObj* obj, int32_t* sizes, int32_t* n_groups);
void visg_obj_free(VisgObj* obj);
/* Mesh::scale (about the vertex mean), Mesh::translate and Mesh::rotation (degrees,
 * axis 0 = x, 1 = y, 2 = z, about the vertex mean) of Mesh.cpp:41-99, in place on
 * n x 3 positions: the transforms the reference's demo applies to its garment and
 * body (main.cpp:24-32). */
int visg_mesh_scale(float* xyz, int32_t n, float s);
int visg_mesh_translate(float* xyz, int32_t n, float dx, float dy, float dz);
int visg_mesh_rotate(float* xyz, int32_t n, float angle_degrees, int32_t axis);

/* ======================================================================== */
/* Body LBVH build that allocates no device memory.                           */
/* ======================================================================== */
/* No counterpart in the reference (its BVHAccel cudaMallocs in every build).
 *
 * For callers that cannot call cudaMalloc themselves or let a library do it: a
 * host application whose own pool allocator owns the device memory, code running
 * where an allocation would synchronise the device at the wrong moment, or a
 * plugin that must not grow the process's memory after start-up.  The caller
 * passes the body in device memory and the output arrays; every temporary of the
 * build lives in one static device array of VISG_NOALLOC_SCRATCH_BYTES, reserved on
 * every GPU that loads the library until the process exits.  The call makes no
 * allocation of any kind.
 *
 *   d_xyz / d_normals   n_vertices*3 floats (normals may be NULL: no thickness push)
 *   d_tris              n_tris*3 vertex indices, each < n_vertices; checked on the device:
 *                       an index out of range is never used to read a vertex, and the
 *                       call's result is then reported as failed (*d_n_leaves = -1)
 *   outputs (device):   d_sorted_codes[n_tris], d_sorted_tris[n_tris] — the first T'
 *                       entries are the de-duplicated Morton order;
 *                       d_child_a/d_child_b[n_tris-1] — the first T'-1 entries are the
 *                       radix tree's links in the reference's encoding (as
 *                       visg_export_lbvh returns them); d_n_leaves[1] = T', or -1 if a
 *                       bounded device wait gave up or an index was out of range (the
 *                       other outputs are then undefined).
 * Limits: n_vertices <= VISG_NOALLOC_MAX_VERTICES, n_tris <= VISG_NOALLOC_MAX_TRIS;
 * larger bodies return VISG_ERR_INVALID_ARG.  Asynchronous on `cuda_stream`.  The
 * first call on a device looks up the static array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  All calls
 * share the array: calls whose GPU work overlaps (other streams, other threads) race. */
#define VISG_NOALLOC_MAX_VERTICES 32768
#define VISG_NOALLOC_MAX_TRIS 32768
#define VISG_NOALLOC_SCRATCH_BYTES (9u * 1024u * 1024u)
/* Self-test of the device-side failure detection: runs, on the current device, one
 * kernel that waits on an mbarrier phase nothing completes (the wait of the step's
 * shared-memory staging ring), one that looks back at a radix-sort status word
 * nothing publishes (the wait of the LBVH's radix passes), and one that waits at a
 * grid barrier for CTAs that never arrive (the wait between the LBVH build's
 * phases).  Each wait is bounded and must give up, record the timeout and return;
 * *gave_up gets bit 0 for the first, bit 1 for the second, bit 2 for the third
 * (7 = all behaved).  Returns VISG_OK when the device is still usable afterwards.
 * Takes about two seconds (the staging wait's and the grid barrier's limits).  No
 * counterpart in the reference. */
int visg_selftest_bounded_waits(int32_t* gave_up);
/* Self-test of the step's exact arithmetic: the zero-damping spring sum evaluates two
 * springs per packed (f32x2) operation and takes each spring's length and its
 * reciprocal from its own correctly rounded square root and reciprocal (Newton
 * corrections of the hardware approximations) on [2^-100, 2^100), the intrinsics
 * outside.  This runs that code on every float of the range, on the current device,
 * against __fsqrt_rn and __frcp_rn(__fsqrt_rn(.)): *checked floats, *mismatches
 * (must be 0).  Takes well under a second.  No counterpart in the reference. */
int visg_selftest_exact_math(uint64_t* checked, uint64_t* mismatches);

int visg_lbvh_build_noalloc(const float* d_xyz, const float* d_normals, int32_t n_vertices,
                            const uint32_t* d_tris, int32_t n_tris, float thickness, float box_depth,
                            uint32_t* d_sorted_codes, int32_t* d_sorted_tris,
                            int32_t* d_child_a, int32_t* d_child_b, int32_t* d_n_leaves,
                            void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* VISG_SIM_H */
