/*
 * morgana_gpu.h -- C ABI of libmorgana_gpu.so, the GB300 (sm_103a) finite-element
 * operator path: P1/P2 tetrahedral element matrices -> CSR -> SpMV / CG.
 *
 * The reference (morganaPublic) exposes this path as a compile-time C++ template
 * API with no FFI; every entry point below names the reference interface it
 * replaces (paths relative to the morganaPublic checkout).
 *
 * Conventions
 *  - Every call returns mg_status (0 = MG_OK).  Nothing aborts or exits; the text
 *    of the last error on the calling thread is available from mg_last_error().
 *  - Indices are 0-based (the reference's gid - 1, as exported to Epetra with
 *    index base 0: src/morganaContainer/pMapGlobalManip.cpp:231-252).
 *  - "d_" arguments are device pointers on the handle's device; "h_" arguments
 *    are host pointers, copied in or out inside the call.
 *  - stream: a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Handles own their device memory, on the device that was current at their
 *    first GPU use; calls on a handle with another device current fail with
 *    MG_ERR_INVALID_ARG.  One handle per host thread; a handle may be shared
 *    between threads only under external locking (the first-use uploads are
 *    locked, the calls themselves are not).
 *  - There is no CPU fallback: a call that cannot run on the GPU fails.
 */
#ifndef MORGANA_GPU_H
#define MORGANA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int mg_status;
enum {
  MG_OK = 0,
  MG_ERR_INVALID_ARG = 1,
  MG_ERR_CUDA = 2,
  MG_ERR_ALLOC = 3,
  MG_ERR_BAD_MESH = 4,       /* detJ <= 0, node id out of range, duplicate nodes in a tet */
  MG_ERR_NOT_CONVERGED = 5,  /* solver hit its iteration cap */
  MG_ERR_UNSUPPORTED = 6,
  MG_ERR_IO = 7,
  MG_ERR_SIZE = 8            /* a size above a documented limit */
};

/* P2 edge numbering rule (src/morganaGeometry/connect3d.hpp:417-491 +
   src/morganaContainer/pVectGlobalManip.hpp). */
enum {
  MG_EDGES_LEX = 0,   /* pMapItem: edges sorted by (min node, max node), :414-486 */
  MG_EDGES_FIRST = 1  /* pMapItemShare on one rank: first appearance in the element x
                         local-edge loop, :498-578 + traitsConnectOptimization.hpp:96-119 */
};

/* Bilinear forms (src/morganaOperators). */
enum {
  MG_OP_STIFF_KAPPA = 0, /* opEL3dA: kappa_e grad u . grad v  (opEL3dA.hpp:129-165) */
  MG_OP_STIFF_CONST = 1, /* opEL3dF: c grad u . grad v        (opEL3dF.hpp:102-133) */
  MG_OP_MASS = 2,        /* opEL3dG: u v                      (opEL3dG.hpp:83-108)  */
  MG_OP_MASS_COEFF = 3   /* opEL3dM: kappa_e u v              (opEL3dM.hpp:129-158) */
};

/* Value precision of an assembled operator / vector.
   MG_F64: double values; the assembly computes them in double-word FP32
     arithmetic (two floats per number, ~48-bit significand, FP64-accurate to
     1e-12) while element-matrix scales (coefficient x geometry) stay within
     2^-96 .. 2^112 in magnitude; outside that range it records a failure that
     mg_plan_status reports (MG_ERR_UNSUPPORTED).
   MG_F32: float values, FP32 arithmetic.
   MG_F64_NATIVE: double values assembled in native FP64 arithmetic (the full
     FP64 range; bound by the FP64 pipe, several times slower).  Every other
     entry point treats it as MG_F64. */
enum { MG_F64 = 0, MG_F32 = 1, MG_F64_NATIVE = 2 };

/* Quadrature: the reference's linearTetra STANDARD cards
   (src/morganaIntegrator/intStaticCards.cpp:707-991) plus the published 11-point
   degree-4 rule of Keast (1986), which the reference does not have. */
enum { MG_QUAD_1 = 1, MG_QUAD_4 = 4, MG_QUAD_11 = 11, MG_QUAD_15 = 15, MG_QUAD_64 = 64 };

/* Preconditioners for the CG solvers. */
enum { MG_PREC_NONE = 0, MG_PREC_JACOBI = 1 };

typedef struct mg_mesh mg_mesh;
typedef struct mg_plan mg_plan;

typedef struct {
  int64_t n_nodes;
  int64_t n_elements;
  int64_t n_edges;
  int64_t ndof;
  int32_t order;      /* 1 or 2 */
  int32_t edge_rule;  /* MG_EDGES_* */
  double min_det;     /* smallest detJ over the reference vertices of every tet */
} mg_mesh_info;

typedef struct {
  int32_t iterations;        /* CG iterations (inner iterations summed for refinement) */
  int32_t outer_iterations;  /* refinement steps (0 for plain CG) */
  int32_t converged;
  int32_t reserved;
  double rel_residual;       /* ||b - A x||_2 / ||b||_2 at exit, FP64 operator
                                (b = 0: the absolute residual ||A x||_2) */
  double seconds;            /* device time of the solve (CUDA events) */
} mg_cg_info;

/* ---------------------------------------------------------------- mesh -- */

/* Builds a mesh from node coordinates (n_nodes x 3) and tetrahedra
   (n_elements x 4, 0-based node ids), numbers edges with edge_rule, and sets up
   the P1 (order 1) or P2 (order 2) dof map.  Node id = position in xyz, element
   order = position in conn, as the Gmsh ingest does.
   Replaces: meshInit3d::gmMesh_to_stdB (src/morganaGeometry/meshInit3d.hpp:485-690)
   with connect3d::buildConnectivity (connect3d.hpp:355-694),
   meshDoctor3d::checkJacobian (meshDoctor3d.hpp:195-227) and
   dofMapStatic3d::startup (src/morganaFields/dofMapStatic3d.hpp:420-560).
   Returns MG_ERR_BAD_MESH when a tet has detJ <= 0 at a reference vertex. */
mg_status mg_mesh_create(mg_mesh** out, int64_t n_nodes, const double* h_xyz, int64_t n_elements,
                         const int32_t* h_conn, int32_t order, int32_t edge_rule);
/* The same mesh with the P2 edges enumerated and numbered on the GPU (element
   edges as sorted node-pair keys, radix-sorted with their incidence index; LEX
   ids from the run heads, FIRST ids by a second sort on first incidence):
   identical edge table, element-to-edge table and dof map.  Needs a device;
   waits for its own work on `stream`.  Up to 2^31 edge incidences (6 E). */
mg_status mg_mesh_create_device(mg_mesh** out, int64_t n_nodes, const double* h_xyz, int64_t n_elements,
                                const int32_t* h_conn, int32_t order, int32_t edge_rule, void* stream);

/* Loads a Gmsh 2.x ASCII mesh: node id = line order in $Nodes (the file's own
   node label is ignored), tetrahedra = element type 4 in file order; the
   triangles (type 2) are kept for mg_mesh_export_triangles.
   Replaces: loadMesh::gmMeshParallel, 3d (src/morganaFile/loadMesh.hpp:2065-2330). */
mg_status mg_mesh_load_gmsh(mg_mesh** out, const char* path, int32_t order, int32_t edge_rule);
/* The Gmsh file's triangles (element type 2), file order: h_tris (n x 3
   0-based node ids, as written) and h_geo_ids (n: the 2nd tag, the geoId
   loadMesh::gmMeshParallel gives the boundary elements,
   src/morganaFile/loadMesh.hpp:2248-2290).  Selecting those of some geoIds and
   passing them to mg_lagrange_build is the reference's test-field geoId
   filter.  n_tris receives the count (0 for meshes not read from Gmsh); the
   arrays may be NULL. */
mg_status mg_mesh_export_triangles(const mg_mesh* mesh, int64_t* n_tris, int32_t* h_tris, int32_t* h_geo_ids);

mg_status mg_mesh_destroy(mg_mesh* mesh);
mg_status mg_mesh_get_info(const mg_mesh* mesh, mg_mesh_info* info);

/* Element -> global dof table (n_elements x nb, nb = 4 or 10), local order
   vertices 1..4 then edges 1..6.
   Replaces: feStaticInterface3d::feIndicesLG (src/morganaFields/feStaticInterface3d.hpp:389-408)
   via dofMapStatic3d::mapListG (dofMapStatic3d.hpp:589-662), minus 1. */
mg_status mg_mesh_export_dofs(const mg_mesh* mesh, int32_t* h_elem_dofs);

/* Edge table: h_edge_nodes (n_edges x 2) = node ids of each global edge, and
   h_elem_edges (n_elements x 6) = global edge of each local edge.
   Replaces: connect3d::getElementToEdge / mesh3d::getEdges (connect3d.hpp:417-491). */
mg_status mg_mesh_export_edges(const mg_mesh* mesh, int32_t* h_edge_nodes, int32_t* h_elem_edges);

/* Node coordinates and connectivity as loaded (for Gmsh ingest checks). */
mg_status mg_mesh_export_geometry(const mg_mesh* mesh, double* h_xyz, int32_t* h_conn);

/* --------------------------------------------------------------- pattern -- */

/* Builds the CSR sparsity pattern (union of element couplings, explicit zeros
   kept, sorted columns) and the element order of the GPU assembly (a Morton
   curve of the element centroids).  The first GPU use of the plan uploads it
   and builds the assembly's block map (P1) or slot map (P2) on the device.
   Replaces: the pattern half of traitsMatrixBuilder::buildEpetraCrs / numEntPerRow
   (src/morganaFiniteElements/traitsMatrixBuilder.hpp:363-544). */
mg_status mg_pattern_build(mg_mesh* mesh, mg_plan** out);
/* The same plan built on the GPU: the CSR pattern (element couplings as
   64-bit keys, radix-sorted and de-duplicated on the device), the element order
   (Morton keys radix-sorted) and the block / slot map, identical to the host build's
   arrays.  The plan is device-resident on return.  Needs a device; waits for
   its own work on `stream`.  Up to 2^31 element couplings (E nb^2), else
   MG_ERR_SIZE.
   Replaces: the same pattern half of buildEpetraCrs. */
mg_status mg_pattern_build_device(mg_mesh* mesh, mg_plan** out, void* stream);
mg_status mg_plan_destroy(mg_plan* plan);
mg_status mg_pattern_info(const mg_plan* plan, int64_t* ndof, int64_t* nnz);

/* rowptr (ndof + 1) and colind (nnz) as int32, 0-based. */
mg_status mg_pattern_export(const mg_plan* plan, int32_t* h_rowptr, int32_t* h_colind);

/* Device copies owned by the plan (valid until mg_plan_destroy). */
mg_status mg_pattern_device(const mg_plan* plan, const int32_t** d_rowptr, const int32_t** d_colind);

/* Slot map of the two-pass GPU assembly of P2 plans (no reference counterpart:
   the reference inserts element blocks into Epetra one by one; P1 plans use the
   block map below, and these calls return MG_ERR_UNSUPPORTED for them).  The
   operators are symmetric, so the
   assembly sums each diagonal and upper CSR entry once and writes it to the entry
   and to its mirror.  These entries are laid out in groups of 32 (one per warp of
   the gather) in the order of (row / rows_per_block, off-diagonal, CSR position):
   per block of rows its diagonal entries, then its other upper entries; entry t
   is written to h_uslot[t] and h_umirror[t] (the same on the diagonal).  Group g holds L = (h_goff[g+1] - h_goff[g]) / 32 rows of sources:
   lane l's j-th source is h_src[h_goff[g] + 32 j + l], 0xffffffff past the end
   of its list.  An entry's sources are the element-matrix entries of every
   element holding both dofs, in ascending Morton position p of the element
   (h_elem_order[p] = element id); a source is p * nunique + u (elem_major = 1,
   P1) or u * n_elem + p (P2), u the upper-triangle index of the element's local
   pair (i <= j, row-major).  Both calls make the plan device-resident (they need
   a device). */
typedef struct {
  int64_t n_upper;    /* diagonal and upper CSR entries */
  int64_t n_groups;   /* groups of 32 of them */
  int64_t n_diag;     /* diagonal entries (the first groups) */
  int64_t n_contrib;  /* sources summed, padding excluded */
  int64_t n_src;      /* length of the source array, padding included */
  int64_t n_elem;
  int32_t nunique;    /* unique entries of an element matrix: 10 (P1), 55 (P2) */
  int32_t elem_major; /* element-matrix layout of the sources (see above) */
  int32_t rows_per_block;
  int32_t reserved;
} mg_slot_map_info;

mg_status mg_plan_slot_map_info(mg_plan* plan, mg_slot_map_info* info);
/* h_elem_order: n_elem; h_goff: n_groups + 1; h_uslot, h_umirror: n_upper;
   h_src: n_src (any may be NULL). */
mg_status mg_plan_export_slot_map(mg_plan* plan, int32_t* h_elem_order, int32_t* h_goff, int32_t* h_uslot,
                                  int32_t* h_umirror, uint32_t* h_src);
/* Block map of the one-pass GPU assembly of P1 plans (no reference counterpart;
   P2 plans use the slot map above, and these calls return MG_ERR_UNSUPPORTED for
   them).  The elements, in Morton order p, form blocks of elems_per_block
   consecutive positions, one CTA each: the CTA computes its elements' matrices
   into shared memory, then sums its block's part of every diagonal and upper CSR
   entry.  An upper entry's sources are the element-matrix entries (p, u) of every
   element holding both of its dofs, ascending p; a run is a maximal stretch of
   them in one block.  An entry with one run is complete and written by its
   block; the others are shared, their runs j = 0, 1, .. in ascending block each
   written to a partial-sum slot, and summed in that order by a second kernel.
   Block b's runs form the groups h_bgrp[b] .. h_bgrp[b+1] of 32 lanes, the
   longest runs first (lengths of 63 and more tied; equal lengths in CSR order).
   Group g
   holds L = (h_goff[g+1] - h_goff[g]) / 32 rows of local sources: lane l's j-th
   source is h_src[h_goff[g] + 32 j + l] = (p - b elems_per_block) nunique + u,
   elems_per_block nunique past the end of its run.  Its output (two int32 per
   lane, h_out[2 (32 g + l)] and [+1]) is (CSR entry, mirror entry) for a complete
   entry, (-1 - q, 0) for partial-sum slot q, (INT32_MIN, 0) for an empty lane.
   The shared entries, sorted by their number of runs (most first; 63 and more
   tied; then CSR order), form groups of 32: group g's slots are
   h_sgoff[g] + 32 j + l, j < (h_sgoff[g+1] - h_sgoff[g]) / 32 (run j of lane l's
   entry; slots past its last run stay zero), and lane l writes its sum to
   h_sout[2 (32 g + l)] and [+1] (INT32_MIN for an empty lane).  Both calls make
   the plan device-resident (they need a device). */
typedef struct {
  int64_t n_upper;          /* diagonal and upper CSR entries */
  int64_t n_contrib;        /* sources summed */
  int64_t n_blocks;         /* element blocks (CTAs) */
  int64_t n_groups;         /* groups of 32 runs */
  int64_t n_src;            /* length of the local-source array, padding included */
  int64_t n_runs;
  int64_t n_shared;         /* entries with sources in more than one block */
  int64_t n_shared_groups;  /* groups of 32 of them */
  int64_t n_partial;        /* partial-sum slots, padding included */
  int64_t n_elem;
  int32_t nunique;          /* unique entries of an element matrix: 10 */
  int32_t elems_per_block;
} mg_block_map_info;

mg_status mg_plan_block_map_info(mg_plan* plan, mg_block_map_info* info);
/* h_elem_order: n_elem; h_bgrp: n_blocks + 1; h_goff: n_groups + 1; h_src: n_src;
   h_out: 64 n_groups; h_sgoff: n_shared_groups + 1; h_sout: 64 n_shared_groups
   (any may be NULL). */
mg_status mg_plan_export_block_map(mg_plan* plan, int32_t* h_elem_order, int32_t* h_bgrp, int32_t* h_goff,
                                   uint16_t* h_src, int32_t* h_out, int32_t* h_sgoff, int32_t* h_sout);
/* The Morton element order alone (host copy; no device needed). */
mg_status mg_plan_export_elem_order(const mg_plan* plan, int32_t* h_elem_order);

/* ------------------------------------------------------------- assembly -- */

/* Assembles the CSR values of one bilinear form into d_values (nnz entries of
   double for MG_F64 or float for MG_F32).  coeff: per-element kappa (device,
   n_elements doubles) for MG_OP_STIFF_KAPPA / MG_OP_MASS_COEFF, else ignored;
   c: the constant of MG_OP_STIFF_CONST.  Deterministic: the same inputs give
   the same bits on every call.  Two assemblies on one plan must not overlap on
   the GPU (other streams): they share the plan's work arrays -- P1: the partial
   sums of the block map (8 bytes per slot, allocated with the plan's device
   state); P2: the element-matrix array (55 x n_elem entries of 8 bytes,
   allocated by the first assembly -- make that call before any stream capture).
   Replaces: the value half of matrixBuilder<localMatrixEL3d<...>>::buildEpetraCrs
   (traitsMatrixBuilder.hpp:363-441) with integratorOEL3d_STD::integration
   (src/morganaIntegrator/integratorOEL3d_STD.hpp:106-137). */
mg_status mg_assemble(mg_plan* plan, int32_t op, const double* d_coeff, double c, int32_t quad,
                      int32_t prec, void* d_values, void* stream);

/* Synchronises the device and reports a failure recorded by an earlier
   asynchronous assembly on this plan: MG_ERR_INVALID_ARG when the coefficient
   array held NaN or Inf,
   MG_ERR_UNSUPPORTED when an MG_F64 assembly met element-matrix scales outside
   its double-word range (assemble with MG_F64_NATIVE, or rescale the
   coefficient by a power of two).  Clears the record.  No reference counterpart (the reference asserts). */
mg_status mg_plan_status(mg_plan* plan);

/* Host-buffer form of mg_assemble, the call an Epetra/Tpetra adapter makes:
   copies h_coeff in, assembles, copies the nnz values out to h_values. */
mg_status mg_assemble_host(mg_plan* plan, int32_t op, const double* h_coeff, double c, int32_t quad,
                           int32_t prec, void* h_values, void* stream);

/* Load vector b_i = sum_e s_e int_e f_h phi_i (f_h the nodal P1/P2 field d_field,
   or 1 when d_field is NULL; s_e = d_elem_scale[e] or 1 when NULL), written to
   d_b (ndof doubles).  Element vectors in double-word arithmetic (FP64-accurate
   at any scale of s and f), then one FP64 sum per dof in a fixed order:
   deterministic, no atomics.  The first call on a plan builds the dof-to-slot
   map (4 bytes per element-vector entry), a work buffer of 8 bytes per entry
   and the element-geometry cache (80 bytes per element) on the device, and
   waits for them: make that first call before capturing a CUDA graph.
   Replaces: vectorBuilder<localVectorEL3d<fnEL3dA|fnEL3dB>>::buildEpetraVector
   (src/morganaFiniteElements/traitsVectorBuilder.hpp:214-274). */
mg_status mg_assemble_rhs(mg_plan* plan, const double* d_field, const double* d_elem_scale,
                          int32_t quad, double* d_b, void* stream);

/* Build addition (the reference imposes Dirichlet data with Lagrange
   multipliers, src/morganaFiniteElements/localMatrixLA3d.hpp:292-322): symmetric
   elimination of the dofs with d_mask[i] != 0 -- their rows and columns are
   zeroed, the diagonal set to 1, and d_b (if not NULL) zeroed there. */
mg_status mg_apply_dirichlet(mg_plan* plan, const uint8_t* d_mask, int32_t prec, void* d_values,
                             double* d_b, void* stream);

/* ---------------------------------------------------------------- solve -- */

/* y = A x with the plan's pattern and d_values; x, y in the value precision.
   Replaces: Epetra_CrsMatrix::Apply as consumed by Belos / ML
   (src/morganaTrilinos/belosBlockCG.hpp:53-73, epetraOperatorSum.cpp:117-128). */
mg_status mg_spmv(mg_plan* plan, int32_t prec, const void* d_values, const void* d_x, void* d_y,
                  void* stream);

/* FP64 preconditioned CG on the FP64 operator: stops when
   ||b - A x||_2 <= rtol ||b||_2 (recursive residual) or after maxit iterations
   (MG_ERR_NOT_CONVERGED).  d_x holds the initial guess on entry.
   Replaces: belosBlockCG::solve (src/morganaTrilinos/belosBlockCG.hpp:46-82),
   block size 1. */
mg_status mg_cg_solve(mg_plan* plan, const double* d_values, const double* d_b, double* d_x,
                      double rtol, int32_t maxit, int32_t precond, mg_cg_info* info, void* stream);

/* Mixed-precision solve: one Jacobi-preconditioned CG sequence on the FP32
   operator with FP32 vectors and FP64 dot products, anchored to FP64 by
   reliable updates.  Whenever the FP32 recursive residual has dropped by the
   factor inner_rtol since the last anchor (or reaches the target), the FP32
   correction is added to the FP64 solution, r = b - A64 x is recomputed in FP64
   and replaces the FP32 residual; the search direction is kept, so the Krylov
   sequence is not restarted.  Stops when ||b - A64 x||_2 <= rtol ||b||_2 (true
   FP64 residual).  max_outer bounds the number of FP64 anchors, max_inner the
   FP32 iterations in total.  Useful inner_rtol: 1e-3 .. 0.5 (1e-2 works well);
   smaller values are raised to 1e-3, because the FP32 recursion drifts from the
   true residual over more than ~3 decades.  mg_cg_info.iterations counts FP32 iterations,
   outer_iterations the anchors.  Build addition (no reference counterpart);
   same role as mg_cg_solve. */
mg_status mg_cg_refined(mg_plan* plan, const double* d_values64, const float* d_values32,
                        const double* d_b, double* d_x, double rtol, int32_t max_outer,
                        int32_t max_inner, double inner_rtol, int32_t precond, mg_cg_info* info,
                        void* stream);

/* FP64 preconditioned CG that allocates nothing: no cudaMalloc, cudaFree,
   event, graph or pinned buffer.  No counterpart in the reference; it serves
   callers that cannot allocate device memory in the solve -- a host code whose
   device memory belongs to another allocator (a caching allocator such as
   PyTorch's, or an arena sized at start-up), or a time-stepping loop that must
   not take the implicit device synchronisation of cudaMalloc/cudaFree.  Same
   arguments, iteration and stopping rule as mg_cg_solve.
   Its work space (five vectors and the reduction scalars) is a fixed 16 MiB
   array in the library's device memory, held by every GPU that loads the
   library until the process exits; ndof is limited to MG_CG_NOALLOC_MAX_NDOF
   (larger plans get MG_ERR_SIZE).  The plan must already be resident on the
   device (any earlier GPU call on it, e.g. mg_assemble), else MG_ERR_INVALID_ARG.
   The first call on a device looks up the array's device address; make that
   first call before any stream capture.  The plan's device must be the
   current device (else MG_ERR_INVALID_ARG).  All calls share the one array: calls
   that overlap on the GPU (other streams, other host threads) race and must be
   serialised by the caller.  Each call re-initialises what it reads. */
#define MG_CG_NOALLOC_MAX_NDOF 400000
mg_status mg_cg_solve_noalloc(mg_plan* plan, const double* d_values, const double* d_b, double* d_x,
                              double rtol, int32_t maxit, int32_t precond, mg_cg_info* info, void* stream);

/* ------------------------------------------------------------- adjoint -- */

/* Build addition: per-element gradient of J(kappa) for the P0 coefficient of
   MG_OP_STIFF_KAPPA, d_grad[e] = -lambda_e^T Khat_e u_e, with Khat_e the
   element stiffness at kappa_e = 1, u the state and lambda the adjoint
   solution (ndof doubles each).  FP64-accurate at any scale of u and lambda.
   The first call on a plan (or the first mg_assemble_rhs) builds the plan's
   element-geometry cache (80 bytes per element on the device) and waits for
   it: make that first call before capturing a CUDA graph. */
mg_status mg_adjoint_grad(mg_plan* plan, const double* d_u, const double* d_lambda, int32_t quad,
                          double* d_grad, void* stream);

/* ------------------------------------------- boundary multipliers -- */

/* Dirichlet data the reference way: P0, P1 or P2 Lagrange multipliers on boundary
   triangles, coupled to the field by opLA3dA (u . q over each boundary face),
   and the saddle system [K B^T; B 0].  FP64 throughout: the boundary work is
   O(n^2) against the O(n^3) of the volume operator. */
typedef struct mg_lagrange mg_lagrange;

/* Triangle quadrature cards of the face operator, by point count: the
   reference's STANDARD linearTriangle cards of precision 1..4
   (src/morganaIntegrator/intStaticCards.cpp:176-300). */
enum { MG_FACE_QUAD_1 = 1, MG_FACE_QUAD_3 = 3, MG_FACE_QUAD_4 = 4, MG_FACE_QUAD_6 = 6 };

typedef struct {
  int64_t n_faces;        /* boundary faces carrying multipliers */
  int64_t n_multipliers;  /* rows of B */
  int64_t ndof;           /* columns of B (the plan's field dofs) */
  int64_t nnz_b;
  int64_t nnz_saddle;     /* (ndof + n_multipliers) rows */
  int64_t nnz_mtm;        /* entries of B^T B (MG_SADDLE_MTM), else 0 */
  int64_t n_mtm_products; /* products B_li B_lj they sum */
  int64_t n_edge_multipliers; /* P2: multipliers on boundary edges (the last ones), else 0 */
  int64_t nnz_mmt;        /* entries of B B^T (MG_SADDLE_MMT), else 0 */
  int64_t n_mmt_products; /* products they sum */
} mg_lagrange_info;

/* Saddle pattern options of mg_lagrange_build. */
enum {
  MG_SADDLE_LAM_DIAG = 1, /* store the multiplier block's diagonal (setEye on that block) */
  MG_SADDLE_MTM = 2,      /* add B^T B to the field block (setMTM(B, field block)) */
  MG_SADDLE_MMT = 4       /* add B B^T to the multiplier block (setMMT(B, multiplier block)) */
};

/* Scales of the saddle blocks (mg_saddle_assemble): setEye on the field and
   multiplier blocks, setMTM and setMMT. */
typedef struct {
  double eye_field, eye_lam, mtm, mmt;
} mg_saddle_scales;

/* Multiplier space and patterns, on the host (no device needed).
   Boundary faces = faces of exactly one tet (connect3d::getFaceIsBoundary),
   in element then local-face order.  h_tris (n_tris x 3 node ids, any vertex
   order) selects the boundary triangles that carry multipliers, the geoId
   filter of the test field (feStaticField2d with dms2d_geoIdMode); NULL = all
   boundary faces.  Multipliers (the test field of opLA3dA):
   - test_order 1 (fePr2d<1>): the P1 dofs of the selected triangles, one per
     node, numbered by ascending node id (meshDoctor2d::removeUnusedPoints,
     src/morganaGeometry/meshDoctor2d.hpp:339-500, then
     src/morganaFields/dofMapStatic2d.hpp:1166-1380);
   - test_order 0 (fePr2d<0>): one per triangle, numbered in the boundary
     grid's element order: the order of h_tris (the Gmsh triangles, whose ids
     the boundary elements keep: src/morganaGeometry/meshInit3d.hpp:400-430),
     or the face order when h_tris is NULL;
   - test_order 2 (fePr2d<2>): the P1 ones, then one per edge of the selected
     triangles in the boundary grid's edge order
     (src/morganaGeometry/connect2d.hpp:336-451): MG_EDGES_LEX meshes (min
     node, max node) order; MG_EDGES_FIRST meshes the order of first
     appearance over every boundary face (element then local-face order) and
     its edges (0,1), (1,2), (2,0) in faceToPoint vertex order, the order in
     which connect3d stores a face.  This takes the boundary grid to be the
     whole boundary: the reference numbers the edges over the triangles its
     Gmsh file lists (src/morganaGeometry/meshInit3d.hpp:411-428), which is the
     same order when those triangles cover the boundary, as Gmsh writes them.
   B (n_multipliers x ndof): each face inserts its full nt x nb block (nt = 3
   for P1, 1 for P0, 6 for P2), explicit zeros included, as
   traitsMatrixBuilder::buildEpetraCrs does for localMatrixLA3d
   (src/morganaFiniteElements/localMatrixLA3d.hpp:292-322).
   Saddle: [K B^T; B 0] (epetraSaddleAssembler::setDiagMatrix + setSymmMatrix,
   src/morganaTrilinos/epetraSaddleAssembler.cpp), with K the plan's pattern.
   flags: MG_SADDLE_LAM_DIAG adds the diagonal of the multiplier block to the
   pattern (setEye on that block); MG_SADDLE_MTM merges the structural pattern
   of B^T B into the field block (setMTM, whose product EpetraExt builds
   structurally: every pair of entries of a multiplier row couples, zeros
   kept); MG_SADDLE_MMT merges B B^T into the multiplier block (setMMT: every
   pair of entries of a field column couples).
   Errors: MG_ERR_BAD_MESH when a face belongs to more than two tets or a
   selected triangle is not a boundary face; MG_ERR_INVALID_ARG for a repeated
   triangle or a node id out of range; MG_ERR_SIZE above 2^31 - 1 entries.
   The handle keeps a pointer to the plan: destroy it before the plan. */
mg_status mg_lagrange_build(mg_plan* plan, int32_t test_order, int64_t n_tris, const int32_t* h_tris,
                            int32_t flags, mg_lagrange** out);
mg_status mg_lagrange_destroy(mg_lagrange* lg);
mg_status mg_lagrange_get_info(const mg_lagrange* lg, mg_lagrange_info* info);
/* h_lam_node (n_multipliers): node (P1, P2 vertex), selected face (P0, an
   index into the face list) or -1 (P2 edge) of each multiplier; h_face_elem,
   h_face_local (n_faces): the selected faces; any pointer may be NULL. */
mg_status mg_lagrange_export(const mg_lagrange* lg, int32_t* h_lam_node, int32_t* h_face_elem,
                             int32_t* h_face_local);
/* P2: (min node, max node) of each edge multiplier, n_edge_multipliers x 2. */
mg_status mg_lagrange_export_edges(const mg_lagrange* lg, int32_t* h_edge_nodes);
/* CSR of B (n_multipliers + 1, nnz_b) and of the saddle matrix
   (ndof + n_multipliers + 1, nnz_saddle); any pointer may be NULL. */
mg_status mg_lagrange_pattern(const mg_lagrange* lg, int32_t* h_b_rowptr, int32_t* h_b_colind,
                              int32_t* h_s_rowptr, int32_t* h_s_colind);

/* The gather maps the kernels read (for host-side checks of the data flow):
   h_b_src_ptr (nnz_b + 1) and h_b_src (n_faces * nt * nb): B entry k sums the
   face-matrix entries h_b_src[h_b_src_ptr[k] .. h_b_src_ptr[k+1]), each
   (face * nt + test basis) * nb + field basis, in that order; h_s_src (nnz_saddle):
   saddle entry k copies K entry h_s_src[k] (>= 0), B entry -(h_s_src[k] + 1),
   the multiplier diagonal (INT32_MIN) or starts at zero (INT32_MIN + 1: a B^T B
   or B B^T entry outside the K / diagonal pattern).  Any pointer may be NULL. */
mg_status mg_lagrange_export_maps(const mg_lagrange* lg, int32_t* h_b_src_ptr, int32_t* h_b_src,
                                  int32_t* h_s_src);
/* The product blocks, which = MG_SADDLE_MTM (B^T B) or MG_SADDLE_MMT (B B^T):
   entry m sums B[k1] B[k2] over the pairs h_pairs[h_pair_ptr[m] ..
   h_pair_ptr[m+1]) (int32 pairs (k1, k2); ascending multiplier row for B^T B,
   ascending field column for B B^T) and adds into saddle entry h_slot[m].
   Sizes: nnz + 1, 2 x products, nnz.  Any pointer may be NULL. */
mg_status mg_lagrange_export_products(const mg_lagrange* lg, int32_t which, int32_t* h_pair_ptr, int32_t* h_pairs,
                                      int32_t* h_slot);

/* Values of B (nnz_b doubles, device) with the face card quad (MG_FACE_QUAD_*):
   one thread per face computes its nt x nb block, then one thread per entry of
   B sums its blocks' contributions in the reference's insertion order
   (deterministic, no atomics).  The first device call on a handle (this one,
   mg_saddle_assemble, mg_saddle_spmv or mg_lagrange_apply) uploads its tables
   and waits for the copies: make it before capturing a CUDA graph.  The face
   blocks go through one staging buffer of the handle, so calls of this
   function on one handle that overlap on the GPU (other streams or host
   threads) race: serialise them. */
mg_status mg_lagrange_assemble(mg_lagrange* lg, int32_t quad, double* d_b_values, void* stream);
/* mg_lagrange_assemble with the values copied to host memory (nnz_b doubles):
   what buildEpetraCrs hands to Epetra for localMatrixLA3d.  Synchronous. */
mg_status mg_lagrange_assemble_host(mg_lagrange* lg, int32_t quad, double* h_b_values);
/* Saddle values (nnz_saddle doubles, device) from K's values (the plan's CSR)
   and B's: [K + eye_field I + mtm B^T B, B^T; B, eye_lam I + mmt B B^T], the
   scales from `scales` (NULL = all 0).  eye_lam must be 0 unless the pattern
   has the multiplier diagonal (MG_SADDLE_LAM_DIAG), mtm / mmt 0 unless it has
   the product (MG_SADDLE_MTM / MG_SADDLE_MMT).  One thread per product entry
   sums its products in a fixed order and adds the sum to its own saddle entry:
   deterministic, no atomics. */
mg_status mg_saddle_assemble(mg_lagrange* lg, const double* d_k_values, const double* d_b_values,
                             const mg_saddle_scales* scales, double* d_values, void* stream);
/* y = S x on the saddle matrix (ndof + n_multipliers doubles each). */
mg_status mg_saddle_spmv(mg_lagrange* lg, const double* d_values, const double* d_x, double* d_y,
                         void* stream);
/* g = B u (u: ndof doubles, g: n_multipliers doubles): the constraint right-hand
   side of nodal Dirichlet data u. */
mg_status mg_lagrange_apply(mg_lagrange* lg, const double* d_b_values, const double* d_u, double* d_g,
                            void* stream);

/* -------------------------------------------------------------- status -- */
const char* mg_status_string(mg_status status);
const char* mg_last_error(void);
/* Library version string. */
const char* mg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MORGANA_GPU_H */
