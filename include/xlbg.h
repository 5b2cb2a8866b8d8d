/*
 * xlbg.h -- C ABI of the GB300 lattice Boltzmann time-step library (libxlbg.so).
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (cudaStream_t passed as void*), returns an int status (XLBG_OK == 0) and
 * never calls cudaMalloc or cudaFree.  Launches are asynchronous on the given
 * stream; nothing synchronises.  The last error message of the calling thread
 * is available from xlbg_last_error().
 *
 * Field layout is XLB's Warp layout (xlb/grid/warp_grid.py:17-32): a population
 * field is (Q, nx, ny, nz) C-contiguous with nz fastest; 2D fields are
 * (Q, nx, ny, 1).  bc_mask is (1, nx, ny, nz) uint8 (0 fluid, 255 skipped).
 *
 * Each declaration names the XLB interface it replaces (file:line in the XLB
 * source tree).
 */
#ifndef XLBG_H
#define XLBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XLBG_ABI_VERSION 1
#define XLBG_MAX_BC 16
#define XLBG_DIAG_SLOTS 1024

/* status codes */
enum {
  XLBG_OK = 0,
  XLBG_ERR_ARG = 1,         /* null pointer, bad size or out-of-range enum */
  XLBG_ERR_UNSUPPORTED = 2, /* e.g. KBC with D3Q19, shifted store with FP64 compute */
  XLBG_ERR_ALIGN = 3,       /* pointer not aligned to its element size */
  XLBG_ERR_CUDA = 4         /* a CUDA launch or API call failed */
};

/* lattice (xlb/velocity_set/{d2q9,d3q19,d3q27}.py) */
enum { XLBG_D2Q9 = 0, XLBG_D3Q19 = 1, XLBG_D3Q27 = 2 };

/* store form of populations (xlb/precision_policy.py:46-81, plus shifted forms) */
enum {
  XLBG_STORE_F32 = 0,
  XLBG_STORE_F64 = 1,
  XLBG_STORE_F16 = 2,   /* raw FP16, XLB's FP32FP16 / FP64FP16 */
  XLBG_STORE_F16S = 3,  /* FP16 holding (f - w_l) * 2^14 */
  XLBG_STORE_BF16S = 4  /* BF16 holding f - w_l */
};
enum { XLBG_COMPUTE_F32 = 0, XLBG_COMPUTE_F64 = 1 };

/* collision (xlb/operator/collision/bgk.py:30-34, kbc.py:192-296).  XLBG_BGK_PAIR is BGK
   with macroscopic and equilibrium rearranged over opposite-direction pairs (one
   reciprocal for u, shared pair terms): the same equations with fewer operations,
   results equal to XLBG_BGK up to rounding.  XLBG_BGK_SHIFTED is the pair form
   evaluated on deviations from rest, g = S (f - w_l): the stored values of the
   shifted stores (XLBG_STORE_F16S / XLBG_STORE_BF16S; one conversion per pulled
   and per stored value), or f - w_l for XLBG_STORE_F32 (exact on load, one
   rounding on store), all with FP32 compute.  Sums of deviations do not cancel
   the way sums of f ~ w_l do.  XLBG_BGK_SHIFTED_SR is XLBG_BGK_SHIFTED on the
   shifted 16-bit stores with stochastic rounding of every store (cvt.rs; random
   bits from a hash of the cell index and the step's timestep argument, so runs
   are reproducible).  No XLB counterpart for 2, 3 and 4. */
enum { XLBG_BGK = 0, XLBG_KBC = 1, XLBG_BGK_PAIR = 2, XLBG_BGK_SHIFTED = 3, XLBG_BGK_SHIFTED_SR = 4 };

/* boundary-condition kinds (xlb/operator/boundary_condition/bc_*.py) */
enum {
  XLBG_BC_FULLWAY_BB = 1,            /* bc_fullway_bounce_back.py:59-72 */
  XLBG_BC_HALFWAY_BB = 2,            /* bc_halfway_bounce_back.py:67-85 */
  XLBG_BC_EQUILIBRIUM = 3,           /* bc_equilibrium.py:75-86 */
  XLBG_BC_ZOUHE_VELOCITY = 4,        /* bc_zouhe.py:279-313 */
  XLBG_BC_ZOUHE_PRESSURE = 5,        /* bc_zouhe.py:315-343 */
  XLBG_BC_REGULARIZED_VELOCITY = 6,  /* bc_regularized.py:134-169 */
  XLBG_BC_REGULARIZED_PRESSURE = 7,  /* bc_regularized.py:171-202 */
  XLBG_BC_EXTRAPOLATION = 8          /* bc_extrapolation_outflow.py:372-415 */
};

typedef struct {
  int32_t id;     /* uint8 id written into bc_mask, 1..254 */
  int32_t kind;   /* XLBG_BC_* */
  double rho;     /* EquilibriumBC density */
  double u[3];    /* EquilibriumBC velocity (u[2] unused in 2D) */
} xlbg_bc;

/*
 * Static description of a stepper.  Replaces the objects XLB bakes into its
 * Warp kernel at construction (nse_stepper.py:25-56, 245-263): velocity set,
 * precision policy, collision type, grid shape and the BC list.
 */
typedef struct {
  int32_t abi_version; /* XLBG_ABI_VERSION */
  int32_t lattice;     /* XLBG_D2Q9 / XLBG_D3Q19 / XLBG_D3Q27 */
  int32_t store;       /* XLBG_STORE_* */
  int32_t compute;     /* XLBG_COMPUTE_* */
  int32_t collision;   /* XLBG_BGK / XLBG_KBC / XLBG_BGK_PAIR / XLBG_BGK_SHIFTED(_SR) */
  int32_t nbc;         /* entries used in bc[] */
  int64_t nx, ny, nz;  /* grid shape; nz = 1 for 2D */
  xlbg_bc bc[XLBG_MAX_BC];
} xlbg_desc;

/* Library and lattice introspection (host only, no GPU needed). */
int xlbg_abi_version(void);
const char* xlbg_last_error(void);
/* c: q*d int32 (c[l*d + k]), w: q doubles, opp: q int32.  Returns q, or <0. */
int xlbg_lattice_tables(int32_t lattice, int32_t* c, double* w, int32_t* opp);

/*
 * Pack XLB's bool missing_mask (Q, nx, ny, nz) into one uint32 per cell, bit l
 * set when direction l is missing.  Replaces the per-step Q-byte read of the
 * mask in nse_stepper.py:311; called once at set-up.
 */
int xlbg_pack_missing(const xlbg_desc* desc, const uint8_t* missing_mask, uint32_t* miss_bits, void* stream);

/*
 * One fused time step: pull stream, streaming-step BCs, macroscopic, quadratic
 * equilibrium, collision, collision-step BCs, extrapolation aux data, aux
 * recovery into f0, store into f1.  Replaces
 * IncompressibleNavierStokesStepper.warp_implementation (nse_stepper.py:385-392)
 * and its kernel (:344-382).  omega is the relaxation rate, timestep is kept for
 * signature parity (unused by the built-in BCs, as in XLB).
 *
 * rec_cells/n_rec: linear indices of the cells whose bc id is a ZouHe or
 * Regularized BC (sorted, int64); rec_scratch: n_rec*Q elements of the store
 * type.  Both may be NULL/0 when the BC list has no such BC.  The recovery
 * writes into f0 happen after every pull of the step, which makes the step
 * deterministic where XLB's kernel races (nse_stepper.py:338-342).
 *
 * With a 16-bit store the first call on a device does one-time set-up of the
 * TMA-staged kernel (shared-memory limits, the fault counter's address, see
 * xlbg_device_faults); make that first call before any stream capture.
 */
int xlbg_step(const xlbg_desc* desc, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss_bits,
              const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, int32_t timestep,
              void* stream);

/*
 * n_steps steps with the caller-side swap of XLB's examples
 * (examples/performance/mlups_3d.py:78-80) done inside: step k reads the
 * buffer written by step k-1.  After an odd n_steps the newest state is in
 * f1, after an even n_steps it is in f0.
 */
int xlbg_run(const xlbg_desc* desc, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss_bits,
             const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, int32_t timestep0,
             int32_t n_steps, void* stream);

/*
 * A step that also returns diagnostics of the states it touches, in FP64:
 *   diag[0] = total mass of the OUTPUT state (sum over non-skipped cells of
 *             sum_l f1_l as stored),
 *   diag[1..d] = momentum-exchange force on the no-slip BC with id force_id
 *             evaluated on the INPUT state f0 -- the value XLB's
 *             MomentumTransfer (xlb/operator/force/momentum_transfer.py:92-176)
 *             returns when called on f0 after the previous step's swap.
 * force_id < 0 disables the force.  diag_slots is caller scratch of
 * XLBG_DIAG_SLOTS*4 doubles that must be zero on entry and is left zero.
 */
int xlbg_step_diag(const xlbg_desc* desc, void* f0, void* f1, const uint8_t* bc_mask, const uint32_t* miss_bits,
                   const int64_t* rec_cells, int64_t n_rec, void* rec_scratch, double omega, int32_t timestep,
                   int32_t force_id, double* diag_slots, double* diag, void* stream);

/*
 * xlbg_step_diag without scratch arguments and without any device allocation.
 * No counterpart in XLB: it exists for callers that cannot allocate device
 * memory around a step -- hosts whose own pool owns the device heap and hand a
 * library only the buffers it reads and writes, and loops that must not call
 * cudaMalloc/cudaFree because those can synchronise the device.
 *
 * Its scratch (the reduction slots and the aux-recovery staging) lives in
 * file-scope __device__ arrays of libxlbg.so, about 4 MiB held by every GPU
 * that loads the library until the process exits.  n_rec * Q * store-bytes
 * must not exceed XLBG_NOALLOC_REC_SCRATCH_BYTES (XLBG_ERR_ARG otherwise).
 * The first call on a device looks up the arrays' device addresses
 * (cudaGetSymbolAddress) for the calling thread's current device; make that
 * first call before any stream capture.  A call that finds the device's
 * context changed since (after cudaDeviceReset) looks them up again, as a
 * first call does.  The arrays are shared by all calls on
 * a device: calls whose GPU work may overlap race on them and must be
 * serialised by the caller.  Same results as xlbg_step_diag.
 */
#define XLBG_NOALLOC_REC_SCRATCH_BYTES (4u << 20)
int xlbg_step_diag_noalloc(const xlbg_desc* desc, void* f0, void* f1, const uint8_t* bc_mask,
                           const uint32_t* miss_bits, const int64_t* rec_cells, int64_t n_rec, double omega,
                           int32_t timestep, int32_t force_id, double* diag, void* stream);

/*
 * Momentum-exchange force on one no-slip BC (halfway or fullway bounce-back),
 * replacing MomentumTransfer(no_slip_bc)(f_0, f_1, bc_mask, missing_mask)
 * (xlb/operator/force/momentum_transfer.py:92-176).  At every cell with
 * bc_mask == bc_id whose rest direction is not missing, each missing direction
 * l adds phi_l = 2 f0[opp l] signed by c[opp l] (the no-slip functionals give
 * f_post_stream[l] = f0[opp l] there); per-cell sums in the compute type, the
 * sum over cells in FP64.  missing_mask is XLB's bool (Q, cells) field.
 * diag_slots: XLBG_DIAG_SLOTS x 4 doubles, zero on entry and left zero; force:
 * 4 doubles, [0, F_x, F_y, F_z] (F_z = 0 in 2D).  Asynchronous on stream.
 */
int xlbg_momentum_transfer(const xlbg_desc* desc, const void* f0, const uint8_t* bc_mask, const uint8_t* missing_mask,
                           int32_t bc_id, double* diag_slots, double* force, void* stream);

/*
 * Differentiation.  XLB differentiates its stepper by taping Warp kernels
 * (examples/out_of_core/subroutine/autodiff_stepper_subroutine.py:460-466,
 * segments of examples/out_of_core/autodiff_lbm.py:64-124); these two entry
 * points replace the tape with a recorded segment of states and a hand-written
 * adjoint kernel.  The state of a step is the population field alone: the
 * ZouHe / Regularized prescribed values, which XLB carries from step to step in
 * f_1 slot 0 (nse_stepper.py:318-342), are passed as a separate field aux (one
 * store-type value per cell, read at those BC cells only; NULL allowed when the
 * BC list has no ZouHe / Regularized BC).
 *
 * xlbg_forward_segment: states holds n_steps + 1 consecutive population fields
 * of Q * cells store elements; for j = 0 .. n_steps - 1 it writes state j + 1 =
 * one step of state j, with the results of xlbg_step when f_1 slot 0 holds aux.
 * No aux recovery: state j is not modified.
 */
int xlbg_forward_segment(const xlbg_desc* desc, void* states, int32_t n_steps, const uint8_t* bc_mask,
                         const uint32_t* miss_bits, const void* aux, double omega, void* stream);

/*
 * xlbg_adjoint_segment: the reverse sweep over a recorded segment.  states
 * holds the n_steps input states of the segment's steps (state j is the input
 * of step j, as written by xlbg_forward_segment).  lam_a holds dL/d(state after
 * the last step) on entry; the sweep ping-pongs between lam_a and lam_b and
 * leaves dL/d(state 0) in lam_a when n_steps is even, in lam_b when it is odd.
 * lam_a / lam_b are Q planes of the compute type.
 *
 * bc_cells / n_bc: sorted linear indices of every cell with a non-zero bc id.
 * aux_grad: n_bc compute-type values; at the ZouHe / Regularized cells of the
 * list, dL/d(aux of that cell) summed over the segment's steps is added to it.
 *
 * Supported: FP32 store with FP32 or FP64 compute, FP64 store with FP64
 * compute; BGK (XLBG_BGK and XLBG_BGK_PAIR, same equations) and KBC; every BC
 * kind.  bc_mask must not contain id 255.  Each step is two kernels: every
 * fluid cell pushes the adjoint of its pulled values back along -c (plain
 * stores; the pull is a bijection per direction) while boundary cells zero
 * their push targets, then the listed boundary cells add their whole local
 * adjoint (pushes, own-cell, neighbour and aux terms) atomically.  Replaces the
 * tape's backward pass.
 */
int xlbg_adjoint_segment(const xlbg_desc* desc, const void* states, int32_t n_steps, const uint8_t* bc_mask,
                         const uint32_t* miss_bits, const void* aux, const int64_t* bc_cells, int64_t n_bc,
                         void* lam_a, void* lam_b, void* aux_grad, double omega, void* stream);

/*
 * Test hook: which step kernel the step entry points launch, process-wide.
 * XLBG_KERNEL_AUTO (the default) picks by store, shape and size; the others
 * force a variant the automatic choice takes only on grids too large for a
 * test (64-bit plane offsets, used when Q * cells >= 2^32), or never on a given
 * shape, so that tests can compare every variant with the CPU restatement on
 * small grids.  Not thread-safe with concurrent steps; set it between steps.
 *   XLBG_KERNEL_MARCH       marching kernel (no TMA staging)
 *   XLBG_KERNEL_MARCH_WIDE  marching kernel with 64-bit plane offsets
 *   XLBG_KERNEL_CELL        one-cell-per-thread kernel (64-bit offsets)
 *   XLBG_KERNEL_TMA_WIDE    TMA-staged kernel with 64-bit plane offsets where
 *                           it applies, else the marching kernel with them
 * Returns XLBG_OK, or XLBG_ERR_ARG for an unknown selector.  No XLB counterpart.
 */
enum {
  XLBG_KERNEL_AUTO = 0,
  XLBG_KERNEL_MARCH = 1,
  XLBG_KERNEL_MARCH_WIDE = 2,
  XLBG_KERNEL_CELL = 3,
  XLBG_KERNEL_TMA_WIDE = 4
};
int xlbg_debug_force_kernel(int32_t kernel);

/*
 * Number of thread blocks of the TMA-staged step (16-bit stores) that gave up
 * on a bounded wait since the last reset (0 in normal operation); such a block
 * stores nothing.  Synchronises with the device.  reset != 0 clears the count.
 * Returns the count, or -XLBG_ERR_CUDA.  No XLB counterpart.
 */
int xlbg_device_faults(int reset);

/*
 * f = feq(rho, u) in the store form for every cell (initializers.py:5-20 with
 * quadratic_equilibrium.py:63-82).  rho: (1, cells) and u: (d, cells) in the
 * compute type, or NULL for the uniform values rho0 / u0[d].
 */
int xlbg_equilibrium(const xlbg_desc* desc, const void* rho, const void* u, double rho0, const double* u0, void* f,
                     void* stream);

/*
 * rho (1, cells) and u (d, cells) in the compute type from a population field
 * (xlb/operator/macroscopic/macroscopic.py:39-55).
 */
int xlbg_macroscopic(const xlbg_desc* desc, const void* f, void* rho, void* u, void* stream);

/*
 * Indices boundary masker for one BC: the per-index work of XLB's Warp
 * IndicesBoundaryMasker kernel (xlb/operator/boundary_masker/
 * indices_boundary_masker.py:114-156).  indices: (3, n) int64, row-major (all
 * x, then all y, then all z; z = 0 on a 2D grid), already shifted by any start
 * index.  Indices outside the grid are skipped.  Each in-grid index gets bc_id;
 * direction l is missing where index - c_l leaves the grid; when needs_padding
 * is non-zero and the index is strictly inside the grid (:29-40), every
 * in-grid pull direction instead marks the push neighbour index + c_l: id
 * bc_id, direction l missing.  Replaces the one racy launch over all BCs
 * (:205-218): call it once per BC in list order and a cell that several BCs
 * touch keeps the last one's id, whatever the thread order.
 */
int xlbg_indices_mask(const xlbg_desc* desc, const int64_t* indices, int64_t n, int32_t bc_id, int32_t needs_padding,
                      uint8_t* bc_mask, uint8_t* missing_mask, void* stream);

/*
 * Mesh boundary masker for one BC: replaces MeshBoundaryMasker.warp_implementation
 * (xlb/operator/boundary_masker/mesh_boundary_masker.py:185-236) and its kernel
 * (:150-183).  3D lattices only.  tri: n_tri triangles of 3 float32 vertices
 * (x, y, z), in grid units; desc gives lattice and grid shape (its store,
 * compute and BC fields are not read).  Voxel p of the grid padded by one cell
 * on every side (p = cell index + 1) is solid when its unit box
 * [p - 1, p] meets a triangle; then every cell whose voxel is solid gets id 255
 * and every other cell with a solid neighbour x + c_l (l >= 1) gets bc_id and
 * missing_mask[opp(l)] = 1.  Other cells and directions are not written, so
 * earlier maskers' marks stay.
 *
 * Work list: the padded grid is cut into bricks of brick^3 voxels, numbered
 * (bx * nby + by) * nbz + bz with nb* = ceil((n* + 2) / brick).  Pair q
 * (pair_tri[q], pair_brick[q]) tests triangle pair_tri[q] against the voxels of
 * brick pair_brick[q] that its bounds meet; the list must hold every (triangle,
 * brick) pair where the triangle's bounds meet a voxel of the brick (extra
 * pairs and repeats are harmless, pairs with an index out of range are
 * skipped).  Scratch, both 16-byte aligned: tri_scratch n_tri *
 * XLBG_MESH_TRI_FLOATS floats, solid_scratch XLBG_MESH_SOLID_BYTES(nx, ny, nz)
 * bytes.
 *
 * flags: XLBG_MESH_EDGE_TESTS also applies the projected-edge tests with the
 * edge terms that pre_compute (:64-97) writes when its nested subscript stores
 * take effect; without it those terms are zero, as the stores leave them in a
 * Warp function, and the tests always pass.
 */
#define XLBG_MESH_TRI_FLOATS 39
#define XLBG_MESH_SOLID_BYTES(nx, ny, nz) (((int64_t)((nx) + 2) * ((ny) + 2) * ((nz) + 2) + 15) / 16 * 16)
#define XLBG_MESH_EDGE_TESTS 1
int xlbg_mesh_mask(const xlbg_desc* desc, const float* tri, int64_t n_tri, const int32_t* pair_tri,
                   const int32_t* pair_brick, int64_t n_pairs, int32_t brick, int32_t bc_id, int32_t flags,
                   float* tri_scratch, uint8_t* solid_scratch, uint8_t* bc_mask, uint8_t* missing_mask, void* stream);

/*
 * Mesh renderer: the per-pixel ray cast and shading of the MeshRenderer operator
 * of XLB's out-of-core example (examples/out_of_core/operators/mesh_renderer.py:
 * 81-187): camera and ray as there, closest hit with t < depth[i, j], vertex
 * colours interpolated with the hit's barycentrics, normal-based shading,
 * gamma; RGBA (pixel: height x width x 4 floats) and depth written on a hit
 * only.  XLB takes the hit from Warp's mesh BVH query; here it comes from a
 * walk through a uniform grid of triangle lists (xlbg_tri_grid, built by the
 * caller: cell (cx, cy, cz) spans lo + cell * (cx, cy, cz) .. + cell and is
 * numbered (cx * dims[1] + cy) * dims[2] + cz; cell_tris[cell_start[k] ..
 * cell_start[k + 1]) lists every triangle whose bounds meet cell k, a superset
 * being fine) with the watertight ray-triangle test (Woop, Benthin and Wald,
 * JCGT 2013); among equal t the lowest face index wins.  face_out (optional,
 * height x width int32) receives the hit face or -1.  err_count (one int32)
 * counts list entries skipped as malformed.  points: n_points x 3 floats;
 * indices: n_tri x 3 int32; vertex_colors: n_points x 3 floats.
 */
typedef struct {
  float lo[3];
  float cell[3];
  int32_t dims[3];
  const int32_t* cell_start;
  const int32_t* cell_tris;
} xlbg_tri_grid;

typedef struct {
  float eye[3], target[3], up[3];
  float fov_degrees, ambient_intensity, edge_sharpness, gamma;
} xlbg_camera;

int xlbg_render_mesh(const float* points, int64_t n_points, const int32_t* indices, int64_t n_tri,
                     const float* vertex_colors, const xlbg_tri_grid* grid, const xlbg_camera* camera, int32_t height,
                     int32_t width, float* pixel, float* depth, int32_t* face_out, int32_t* err_count, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* XLBG_H */
