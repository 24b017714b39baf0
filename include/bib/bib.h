/*
 * bib.h -- C ABI of biblbm_gb300, the GB300 (sm_103a) implementation of the
 * coupled immersed-boundary lattice-Boltzmann time step of niclasberg/biblbm.
 *
 * The entry points mirror the three extension points the reference exposes on
 * this path, so that a Palabos / fsi driver (progs/ in the reference) can hand the
 * step to the GPU:
 *
 *   1. Palabos' collide-and-stream offload interface CoProcessor3D<T>
 *      (src/coProcessors/coProcessor3D.h:57-115): addDomain / send / receive /
 *      collideAndStream  ->  bib_lattice_add_domain / _send / _receive /
 *      _collide_and_stream.
 *   2. The fsi data-processor functional ImmersedBoundaryWrapperFunctional3D
 *      (src/fsi/DataProcessors.h:110-139, process() at DataProcessors.hh:94-108)
 *      and the driver step order of progs/capsule_in_shear/capsule_in_shear.cpp:187-227
 *      ->  bib_ibm_step / bib_step.
 *   3. The particle model API: ParticleShapeLibrary::store_mesh
 *      (src/fsi/ParticleShapeFactory.h:26), ImmersedBoundaryDynamics3D::add_particle /
 *      get_particle / compute_total_volume (src/fsi/ImmersedBoundaryDynamics.h:63-113)
 *      ->  bib_shape_store / bib_particle_add / bib_particle_get / bib_total_volume.
 *
 * Conventions
 *  - Every call returns a bib_status: 0 on success, a negative code on failure.
 *    The library never exits or traps (the reference calls exit(-1),
 *    ImmersedBoundaryDynamics.hh:51-54).  bib_last_error() gives the message.
 *  - The caller owns all host buffers; they are copied.  The library owns device
 *    memory.  Handles are small non-negative integers, as CoProcessor3D::addDomain's.
 *  - A context is not thread-safe: use it from one host thread.  Calls are ordered
 *    on the context's CUDA stream; calls that return host data synchronise.
 *  - Lattice fields exchanged with the host are FP64 structure-of-arrays with x
 *    fastest: value(c, x, y, z) = a[c*n + x + nx*(y + ny*z)], n = nx*ny*nz.
 *    Populations are f-bar = f - t_i (Palabos DefaultRoundOffPolicy,
 *    src/latticeBoltzmann/roundOffPolicy.h:72-90) in the reference's D3Q19 order
 *    (src/latticeBoltzmann/nearestNeighborLattices3D.hh:165-197), post-streaming,
 *    i.e. the state Palabos holds between two time steps.
 */
#ifndef BIB_BIB_H
#define BIB_BIB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BIB_ABI_VERSION 1

typedef int32_t bib_status;
enum {
    BIB_OK = 0,
    BIB_EINVAL = -1,       /* bad argument, handle or size */
    BIB_ENOMEM = -2,       /* device or host allocation failed */
    BIB_ECUDA = -3,        /* a CUDA call failed */
    BIB_ENAN = -4,         /* the state contains NaN / Inf */
    BIB_ETIMEOUT = -5,     /* a bounded device wait gave up */
    BIB_ESTATE = -6,       /* call not valid in the current state */
    BIB_EUNSUPPORTED = -7, /* option combination not implemented */
    BIB_EOVERFLOW = -8     /* a fixed-capacity device buffer overflowed (see bib_check_health) */
};

/* population storage on the device.  F64 keeps the reference's arithmetic (the parity path; its
 * collision is FP64-bound on this part, ~1/20 of the F16 step's rate).  F32 collides in FP32 at
 * twice F16's bytes.  F16 stores f-bar times a scale (f16_scale) and collides in FP32: it pays on
 * large lattices, whose step is bound by moving the populations (the 8.4 M-cell channel: FP16 1.27x
 * FP32); on lattices below ~1 M cells the step is bound by its launches and the immersed boundary,
 * FP16 is no faster than FP32 there and its error is two orders larger (64^3 capsule: Taylor
 * deformation error 4.5e-4 against 2.4e-6), so F32 is the better choice there. */
enum { BIB_STORAGE_F64 = 0, BIB_STORAGE_F32 = 1, BIB_STORAGE_F16 = 2 };
/* collision operator */
enum {
    BIB_COLLISION_BGK_GUO_VOF = 0, /* GuoExternalForceVOFDynamics, src/fsi/VariableViscosityDynamics.hh:151-172 */
    BIB_COLLISION_BGK = 1,         /* BGKdynamics, src/basicDynamics/isoThermalDynamics.hh:329-340 */
    BIB_COLLISION_TRT = 2          /* two-relaxation-time (no reference counterpart) */
};
/* wall treatment on a non-periodic axis */
enum {
    BIB_WALL_NONE = 0,
    BIB_WALL_FD_VELOCITY = 1, /* createInterpBoundaryCondition3D velocity walls (y only) */
    BIB_WALL_HALFWAY_BB = 2   /* link-wise halfway bounce-back, optional moving wall */
};
enum { BIB_DIRAC_ROMA = 0, BIB_DIRAC_PESKIN = 1 };
enum {
    BIB_MODEL_CAPSULE_NEOHOOKEAN = 0, /* DeformableCapsuleParticle, src/fsi/DeformableCapsule.hh:60-150 */
    BIB_MODEL_CAPSULE_SKALAK = 1,
    BIB_MODEL_RBC_WLCPOW = 2,         /* RBCParticle, src/fsi/RBCParticle.hh:140-247 */
    BIB_MODEL_SKALAK_BENDING = 3      /* Skalak law + the RBC area / volume / bending terms */
};
enum { BIB_SPREAD_ATOMIC = 0, BIB_SPREAD_DETERMINISTIC = 1 };
/* host layouts of bib_lattice_send / _receive:
 *  SOA_F64         19 arrays of n doubles, x fastest (this library's order)
 *  PALABOS_F64     Palabos static-cell wire order: x-major, z fastest, 23 doubles per cell
 *                  (19 f-bar + 4 external scalars: force, phase), blockLattice3D.hh:671-689
 *  COPROCESSOR_F64 CoProcessor3D::send order: x-major, z fastest, 19 f-bar per cell
 *                  (coProcessor3D.h:80-91) */
/* per-cell dynamics, defineDynamics(lattice, domain, new BounceBack / NoDynamics), core/dynamics.h:559-600 */
enum { BIB_CELL_FLUID = 0, BIB_CELL_BOUNCE_BACK = 1, BIB_CELL_NO_DYNAMICS = 2 };

/* collide-and-stream kernel choice (no reference counterpart: a GPU tuning knob) */
enum { BIB_KERNEL_AUTO = 0, BIB_KERNEL_ROWS = 1, BIB_KERNEL_STAGED = 2 };

enum { BIB_LAYOUT_SOA_F64 = 0, BIB_LAYOUT_PALABOS_F64 = 1, BIB_LAYOUT_COPROCESSOR_F64 = 2 };

/* membrane parameter vector, 12 doubles */
enum {
    BIB_P_G = 0, BIB_P_C, BIB_P_NU_S, BIB_P_KB,               /* CapsuleParameters, DeformableCapsule.h:22-31 */
    BIB_P_SHEAR_MODULUS, BIB_P_L0, BIB_P_K_AREA_GLOBAL,       /* RBCParameters, RBCParticle.h:21-58 */
    BIB_P_K_AREA_LOCAL, BIB_P_K_VOLUME, BIB_P_VOL_DESIRED, BIB_P_K_BEND, BIB_P_THETA0,
    BIB_P_COUNT
};

typedef struct bib_ctx bib_ctx;

typedef struct {
    int32_t device; /* CUDA device ordinal */
    int32_t flags;  /* reserved, 0 */
} bib_config;

typedef struct {
    int32_t periodic[3];     /* per axis: 1 periodic, 0 walled */
    int32_t collision;       /* BIB_COLLISION_* */
    int32_t storage;         /* BIB_STORAGE_* */
    int32_t wall_y, wall_z;  /* BIB_WALL_* for a non-periodic y / z axis */
    int32_t use_phase;       /* 1: per-cell phase field enters omega (viscosity ratio != 1) */
    int32_t reserved;
    double omega;            /* outer-fluid relaxation frequency (omega1 of the VOF dynamics) */
    double omega_inner;      /* inner-fluid relaxation frequency (omega2) */
    double trt_magic;        /* TRT magic parameter Lambda */
    double wall_u[4][3];     /* velocity of the y-, y+, z-, z+ walls */
    double body_force[3];    /* constant body force added to the force field every step */
    double f16_scale;        /* FP16 storage stores f-bar * scale; 0 selects the default 8192 */
} bib_lattice_params;

typedef struct {
    int32_t dirac;        /* BIB_DIRAC_* */
    int32_t spread_mode;  /* BIB_SPREAD_* */
    double field_offset;  /* location of the velocity field of the reference's data processor: -1 */
} bib_ib_params;

typedef struct {
    int32_t collide_kernel; /* BIB_KERNEL_*: AUTO takes the shared-memory staged kernel where the x-row fits */
    int32_t tile_cells;     /* staged kernel: cells per tile (whole x-rows); 0 = 512 (256 for FP64) */
    int32_t stages;         /* staged kernel: pipeline depth 2..4; 0 = the deepest that keeps the CTAs resident */
    int32_t membrane_block; /* threads per particle of the membrane kernel: 64 .. 512 (power of two), 0 = 256 */
    int32_t force_reset;    /* BIB_FORCE_RESET_*: how the coupled step resets the previous force field */
    int32_t wait_limit_us;  /* staged kernel: bound of each hand-off wait between its warps, in microseconds
                             * (0 = 2 s).  A wait that runs out makes the launch give up and bib_check_health
                             * return BIB_ETIMEOUT; the wait for the kernel's own copies in flight keeps 2 s */
    int32_t withhold_tile;  /* failure testing: 1 + the index of a tile of the staged kernel whose copies its
                             * producer does not issue, so that the consumers' wait for them runs out (0 = none) */
    int32_t reserved[1];
} bib_tuning;
/* DENSE (AUTO's choice): the collide-and-stream reads the previous force field for the velocity and
 * resets it to the body force, 24 bytes per cell streamed.  SPARSE (reduced-precision lattices
 * without phase field, cell types, second-order walls or pipe boundary; others stay dense): the
 * collide-and-stream neither reads nor rewrites the previous field, the interpolation gathers its
 * share at the support nodes and only the nodes the last spreading wrote are reset.  Sparse pays
 * off for dilute suspensions only: on 400 cells of 642 vertices in 512 x 128 x 128 it saved
 * 0.016 ms per step in the collide-and-stream and cost 0.136 ms in the scattered gathers and
 * resets. */
enum { BIB_FORCE_RESET_AUTO = 0, BIB_FORCE_RESET_DENSE = 1, BIB_FORCE_RESET_SPARSE = 2 };

/* ---- context (src/coProcessors/coProcessor3D.h:57-115 lifetime) ---- */
bib_status bib_create(const bib_config* cfg, bib_ctx** out);
void bib_destroy(bib_ctx* ctx);
bib_status bib_sync(bib_ctx* ctx);
size_t bib_last_error(const bib_ctx* ctx, char* buf, size_t len);
const char* bib_status_string(bib_status s);
int32_t bib_abi_version(void);

/* ---- lattice: CoProcessor3D::addDomain / send / receive / collideAndStream ---- */
/* CoProcessor3D::addDomain(nx, ny, nz, omega, handle), coProcessor3D.h:69-74 */
bib_status bib_lattice_add_domain(bib_ctx* ctx, int64_t nx, int64_t ny, int64_t nz, const bib_lattice_params* p,
                                  int32_t* handle);
/* The lattice parameters of a CoProcessor3D domain (coProcessor3D.h:69-74, the omega of its BGK
 * dynamics): collision BIB_COLLISION_BGK (or BIB_COLLISION_BGK_GUO_VOF for blocks that carry a
 * force), the given storage, every axis wrapped periodically (the interface leaves the outer
 * one-cell layer undefined, coProcessor3D.h:105-107), no walls, no body force.  Used by
 * bib/bib_coprocessor3D.h. */
bib_status bib_coprocessor_domain_params(double omega, int32_t storage, int32_t collision, bib_lattice_params* p);
/* defineDynamics with BounceBack / NoDynamics per cell (rbc_in_pipe.cpp:307-310): types is nz x ny x nx
 * BIB_CELL_* values (x fastest); BounceBack nodes swap each population with its opposite instead of
 * colliding, NoDynamics nodes keep theirs; both report zero velocity.  NULL restores the lattice's
 * dynamics everywhere. */
bib_status bib_lattice_set_cell_types(bib_ctx* ctx, int32_t h, const uint8_t* types);
/* The pipe walls of progs/rbc_in_pipe/rbc_in_pipe.cpp:300-318 for a PipeBoundary along x through
 * (y0, z0) (fsi/Boundary.h:132-249).  second_order = 0: BounceBack on the nodes outside the pipe;
 * second_order = 1: GuoRigidWallBoundary (fsi/GuoBoundaryCondition.hh): the outside nodes with a
 * lattice vector crossing the wall are rebuilt after every collide-and-stream from the two fluid
 * nodes along their best-aligned vector (BIB_EUNSUPPORTED if a pipe is too narrow for that).  Both:
 * NoDynamics beyond radius + 1.  Replaces the cell types; bib_lattice_set_cell_types removes them. */
bib_status bib_lattice_set_pipe_walls(bib_ctx* ctx, int32_t h, double y0, double z0, double radius, int32_t second_order);
/* CoProcessor3D::send, coProcessor3D.h:75-91: whole-domain populations from the host in one of
 * the BIB_LAYOUT_* orders (the PALABOS layout also sets the force and phase scalars). */
bib_status bib_lattice_send(bib_ctx* ctx, int32_t h, const void* buf, size_t bytes, int32_t layout);
/* CoProcessor3D::receive, coProcessor3D.h:85-93 */
bib_status bib_lattice_receive(bib_ctx* ctx, int32_t h, void* buf, size_t bytes, int32_t layout);
/* CoProcessor3D::collideAndStream, coProcessor3D.h:94-97 (plus the wall processors) */
bib_status bib_lattice_collide_and_stream(bib_ctx* ctx, int32_t h, int64_t nsteps);
/* initializeAtEquilibrium (core/cell.hh:124-132) from rho (n, may be NULL = 1) and u (3n),
 * then the wall processors once (MultiBlock3D::initialize) */
bib_status bib_lattice_init_equilibrium(bib_ctx* ctx, int32_t h, const double* rho, const double* u);
/* external force scalars (3n): setExternalVector / read back */
bib_status bib_lattice_set_force(bib_ctx* ctx, int32_t h, const double* F);
bib_status bib_lattice_get_force(bib_ctx* ctx, int32_t h, double* F);
/* phase scalar (n, values 0..1), used when use_phase = 1.  With particles the lattice keeps it
 * up to date itself: the membranes are voxelized into it when the particles are first stepped
 * and after every move (ImmersedBoundaryDynamics_voxelization.hh:17-30, 121-161) */
bib_status bib_lattice_set_phase(bib_ctx* ctx, int32_t h, const double* phase);
bib_status bib_lattice_get_phase(bib_ctx* ctx, int32_t h, double* phase);
/* computeVelocity (dataAnalysisWrapper3D.hh:1660): u = j/rho + F/2, wall nodes give the wall velocity */
bib_status bib_lattice_get_velocity(bib_ctx* ctx, int32_t h, double* u);
bib_status bib_lattice_cells(bib_ctx* ctx, int32_t h, int64_t* n);

/* ---- shapes: ParticleShapeLibrary::store_mesh, ParticleShapeFactory.hh:120-137 ---- */
bib_status bib_shape_store(bib_ctx* ctx, const double* xyz, const int64_t* tri, int64_t nv, int64_t nt, int32_t* shape);
/* out[6] = {area, volume, n_links, n_pairs, n_vertices, n_triangles} */
bib_status bib_shape_info(bib_ctx* ctx, int32_t shape, double* out);
/* the shape's tag (ParticleShape::get_tag, ParticleShape.h:64), written by the lightweight output */
bib_status bib_shape_set_tag(bib_ctx* ctx, int32_t shape, const char* tag);

/* ---- RBC shape calibration (progs/common/calibrate_rbc_shape.h) ----
 * bib_rbc_params: create_rbc_params (:72-110) for an RBC on `shape`: L0 = mean link length,
 * vol_desired = the shape's volume, k_area_global / k_area_local = 0.8 / 0.2 of (k_area - 2 G),
 * k_volume = 1000 G / (radius of the rest vertices around the origin), k_bend, theta0 of a closed
 * triangulation; prm receives BIB_P_COUNT values (capsule entries 0).
 * bib_rbc_shrink_volume: shrink_rbc_volume (:12-69) on the GPU: an RBC on `shape` (its rest
 * vertices) with `params` relaxes by RBCParticle::relax_nodes (RBCParticle.hh:318-342) for
 * 2 n_it + 1 iterations while vol_desired ramps from the shape's volume to vol_final over the first
 * n_it; a relaxation whose area turns NaN restarts with the damping doubled (at most 64 times,
 * then BIB_ENAN).  pos_out receives 3 nv doubles, damping_out (optional) the damping used.
 * bib_align_minor_axis: DeformableParticle3D::set_minor_axis_orientation (DeformableParticle3D.hh:
 * 85-144) of the vertices pos (3 nv, in place) of a particle on `shape`: the eigenvector of the
 * tensor of gyration with the smallest eigenvalue is rotated onto dir about the centre of mass. */
bib_status bib_rbc_params(bib_ctx* ctx, int32_t shape, double shear_modulus, double k_area, double k_bend, double* prm);
bib_status bib_rbc_shrink_volume(bib_ctx* ctx, int32_t shape, const double* params, double vol_final, int64_t n_it,
                                 double damping, double* pos_out, double* damping_out);
bib_status bib_align_minor_axis(bib_ctx* ctx, int32_t shape, double* pos, const double* dir);

/* ---- random initial placement (progs/common/create_particles.h:37-93 with
 * ParticlePositionInitializer, src/fsi/ParticlePositionInitializer.hh:17-80), host only ----
 * counts[t] spheres of radius radii[t] per type t, in type order, at uniform positions in the box
 * {x0, x1, y0, y1, z0, z1} (integers, shrunk by the radius), inside the pipe {y0, z0, radius} by the
 * radius when pipe is non-NULL, overlapping no earlier sphere (radii <= max_radius), then one random
 * orientation quaternion {w, x, y, z} per sphere; drawn from the sequence of glibc's rand() after
 * srand(seed), so that the reference's driver gets the same numbers.  pos: 3 per sphere, quat: 4.
 * BIB_EOVERFLOW if a sphere finds no free place within max_tries draws (the reference tries 5e6). */
bib_status bib_initial_distribution(const int64_t* box, const double* pipe, int32_t ntypes, const int64_t* counts,
                                    const double* radii, double max_radius, uint32_t seed, int64_t max_tries,
                                    double* pos, double* quat);

/* ---- growth of the initial distribution (progs/common/create_particles.h:105-212) ----
 * bib_grow_particles: rigid copies (RigidParticle3D, RigidParticle.hh) of the stored shapes
 * shape[k], centred at com[k] with orientation quat[k] ({w, x, y, z}), grow from initial_scale:
 * every rescale_every iterations the scale becomes initial_scale + (1 - initial_scale) it / n_it;
 * each iteration the vertices feel SpringPotential(min_dist, strength) collision forces between
 * particles and, with has_wall, against the PipeBoundary wall (compute_collision_forces with the
 * reference's grid search and wall pass, CollisionForces.h:63-184), and every particle moves as a
 * damped rigid body (RigidParticle3D::move_vertices, RigidParticle.hh:55-101) with the periodic
 * remap of its centre.  The box is the lattice's bounding box (each extent >= 2).  Iterations
 * 0 .. it_end - 1 run on the GPU (n_it + 1 of them: the whole growth); com and quat are updated in
 * place; pos_out / force_out (optional, 3 doubles per vertex in particle order) receive the
 * vertex positions after the last iteration and the collision forces of its force step.  The
 * force and move arithmetic follows the reference's operation order (the forces bit for bit; the
 * rotation's sin / cos are CUDA's).
 * bib_place_particle: the final placement of create_particles (:193-199): the vertices xyz of a
 * particle on `shape` (NULL: the shape's rest vertices) moved by translate(-c), rotate(quat),
 * translate(com) (Transform.hh:28-85), c their centre of mass (DeformableParticle3D::update);
 * host only. */
typedef struct {
    int64_t box[6];            /* x0, x1, y0, y1, z0, z1 */
    int32_t periodic[3];
    int32_t has_wall;
    double wall[3];            /* y0, z0, radius of the pipe (the drivers pass the pipe radius - 1.5) */
    double min_dist, strength; /* SpringPotential: cutoff min_dist in (0, 1] */
    double initial_scale, density, damping;
    int64_t n_it;              /* the scale reaches 1 at iteration n_it (the reference's drivers: 40000) */
    int64_t rescale_every;     /* the reference's drivers: 10 */
    int64_t it_end;            /* in [0, n_it + 1] */
} bib_growth;
bib_status bib_grow_particles(bib_ctx* ctx, const bib_growth* g, int32_t n, const int32_t* shape, double* com,
                              double* quat, double* pos_out, double* force_out);
bib_status bib_place_particle(bib_ctx* ctx, int32_t shape, const double* xyz, const double* com, const double* quat,
                              double* out);

/* ---- immersed boundary: ImmersedBoundaryDynamics3D ---- */
bib_status bib_ib_configure(bib_ctx* ctx, int32_t h, const bib_ib_params* p);
/* ImmersedBoundaryDynamics3D::set_boundary with a PipeBoundary along x through (y0, z0): vertices
 * within the kernel's half support + 1 of the wall interpolate and spread with a blend of the
 * kernel and the 2-point TopHat (interpolate_near_boundary / spread_forces_near_boundary,
 * ImmersedBoundaryDynamics_interpolation.hh:181-230, _forces.hh:192-237), and a move that crosses
 * the wall is reflected (DeformableParticle3D.hh:26-51).  radius <= 0 removes it.  Atomic
 * spreading only. */
bib_status bib_ib_set_pipe_boundary(bib_ctx* ctx, int32_t h, double y0, double z0, double radius);
/* add_particle (ImmersedBoundaryDynamics.hh:500-525): xyz NULL = the rest shape */
bib_status bib_particle_add(bib_ctx* ctx, int32_t h, int32_t shape, int32_t model, const double* params,
                            const double* xyz, int32_t* pid);
bib_status bib_particle_count(bib_ctx* ctx, int32_t h, int32_t* n);
/* shape id, membrane model and vertex count of particle pid: out[0..2] */
bib_status bib_particle_info(bib_ctx* ctx, int32_t h, int32_t pid, int32_t* out);
bib_status bib_particle_get(bib_ctx* ctx, int32_t h, int32_t pid, double* pos, double* vel, double* force);
bib_status bib_particle_set_positions(bib_ctx* ctx, int32_t h, int32_t pid, const double* pos);
/* out[14] = {area, volume, com[3], moment of inertia[9]} (DeformableParticle3D.hh:54-82, 173-272) */
bib_status bib_particle_stats(bib_ctx* ctx, int32_t h, int32_t pid, double* out);
/* all vertex positions (3 * total vertices) and per-particle {area, volume, com[3]} (5 per particle) */
bib_status bib_particles_download(bib_ctx* ctx, int32_t h, double* pos, double* stats);
/* all vertex positions (3 per vertex, particles in order) into the device state without
 * re-building it: the area, volume and centre follow as after a step's move (the centre mapped
 * to the periodic grid, the vertices with it), and a phase field is re-voxelized.  Asynchronous
 * on the context's stream; the host buffer is read before the call returns only when the
 * particles have not been uploaded yet.  Otherwise the copy reads it later: keep the buffer
 * unchanged and allocated until bib_sync (or any call that waits for the stream: receive,
 * downloads, bib_check_health) has returned. */
bib_status bib_particles_upload(bib_ctx* ctx, int32_t h, const double* pos);
/* bib_particles_download without waiting: the copies are queued on the context's stream behind the
 * work issued so far, and slot (0..7) marks their completion.  The host buffers must stay valid (and
 * be pinned for the copy to overlap) until bib_download_wait(ctx, slot) returns; a step issued in
 * between runs while the copy's data are read.  Either pointer may be NULL.  A page-locked stats
 * buffer is written by a small kernel through its mapped address (no copy-engine hand-over between
 * the steps of a step-then-read loop). */
bib_status bib_particles_download_async(bib_ctx* ctx, int32_t h, double* pos, double* stats, int32_t slot);
bib_status bib_download_wait(bib_ctx* ctx, int32_t slot);
bib_status bib_total_vertices(bib_ctx* ctx, int32_t h, int64_t* n);
/* compute_total_volume, ImmersedBoundaryDynamics.hh:559-568 */
bib_status bib_total_volume(bib_ctx* ctx, int32_t h, double* v);
/* ---- interaction forces added to the vertex forces of every IB step (compute_forces,
 * ImmersedBoundaryDynamics_forces.hh:287-302): wall interactions first (add_force_decorator with
 * WallInteraction, ForceDecorator.hh:25-32), then the membrane forces, then particle-particle
 * interactions (add_pp_force with PPPotentialForce, ParticleParticleInteraction.h:24-40, evaluated
 * as CollisionHandler::handle_collision, CollisionForces.h:187-199).  Potentials (Potentials.h):
 * Morse 2 beta strength x (x - 1), x = exp(beta (r0 - d)); spring (r0 - d) strength; both act
 * for d <= r0.  Pair search BIB_PAIR_SEARCH_ALL takes every pair of vertices of different
 * particles within r0 (minimum image on periodic axes).  BIB_PAIR_SEARCH_GRID is the reference's
 * own search (CollisionHandler over a Grid of ~unit cells, CollisionForces.h:63-164, Grid.hh): a
 * cell pairs with 7 of its 13 forward neighbours, so pairs in cells offset by e.g. (+1, -1, 0) are
 * missed; only vertices inside the lattice box enlarged by 1/2 + r0 take part; the terms are
 * accumulated in the reference's order, one potential after the other.  All particle-particle
 * interactions of a lattice use one search.  Particle-particle cutoffs are limited to the delta
 * kernel's half support - 1/2, as in the reference (ImmersedBoundaryDynamics_forces.hh:346-349). ---- */
enum { BIB_POTENTIAL_NONE = 0, BIB_POTENTIAL_MORSE = 1, BIB_POTENTIAL_SPRING = 2 };
enum { BIB_PAIR_SEARCH_ALL = 0, BIB_PAIR_SEARCH_GRID = 1 };
typedef struct {
    int32_t kind;    /* BIB_POTENTIAL_* */
    int32_t search;  /* BIB_PAIR_SEARCH_* (particle-particle interactions; ignored for walls) */
    double r0;       /* Morse r_min / spring min_dist: the cutoff */
    double beta;     /* Morse beta (unused by the spring) */
    double strength; /* Morse strength / spring constant */
} bib_potential;
#define BIB_MAX_WALL_INTERACTIONS 4
#define BIB_MAX_PP_INTERACTIONS 4
/* WallInteraction with ParallelPlatesBoundary(lo, hi) (Boundary.h:305-365) normal to axis 1 (y,
 * the reference's plates) or 2 (z): distance to the nearer plate, force -= phi(dist) outward normal */
bib_status bib_add_wall_interaction(bib_ctx* ctx, int32_t h, int32_t axis, double lo, double hi, const bib_potential* p);
/* WallInteraction on a PipeBoundary along x through (y0, z0) (rbc_in_pipe.cpp:154-163,
 * ForceDecorator.hh:25-32, Boundary.h:158-161, 245-249): a vertex at distance
 * dist = radius - sqrt((y - y0)^2 + (z - z0)^2) <= r0 from the wall gets force -= phi(dist) n,
 * n = (0, y - y0, z - z0) / |.| */
bib_status bib_add_pipe_wall_interaction(bib_ctx* ctx, int32_t h, double y0, double z0, double radius,
                                         const bib_potential* p);
bib_status bib_add_pp_interaction(bib_ctx* ctx, int32_t h, const bib_potential* p);
bib_status bib_clear_interactions(bib_ctx* ctx, int32_t h);

/* ImmersedBoundaryDynamics3D::init (ImmersedBoundaryDynamics.hh:404-412): upload the particles
 * and, on a lattice with a phase field, voxelize them into it.  The first step does this by
 * itself; the call makes the moment explicit (and synchronises). */
bib_status bib_ibm_init(bib_ctx* ctx, int32_t h);
/* One IB step on the current lattice state: velocity at the vertices, forces, spreading
 * into a force field reset to the body force, vertex motion (DataProcessors.hh:104-107). */
bib_status bib_ibm_step(bib_ctx* ctx, int32_t h);
/* steps taken by the lattice (bib_step, bib_ibm_step, collide-and-stream, batch steps); the
 * counterpart of the reference's Time (Time.h:20-35), kept in checkpoints */
bib_status bib_lattice_iteration(bib_ctx* ctx, int32_t h, int64_t* iteration);

/* ---- checkpoints: parallelIO::save / load of the lattice (io/multiBlockWriter3D.cpp:201,
 * io/multiBlockReader3D.cpp:261), save_checkpoint / load_checkpoint of the particles
 * (ImmersedBoundaryDynamics_io.hh:17-158) and the iteration counter, in one versioned binary file
 * per lattice.  Device buffers are stored in their own storage type: a resumed run continues
 * bit for bit (with deterministic spreading).  Load needs a lattice created with the same
 * parameters and a context holding the same shapes under the same ids; it replaces the lattice's
 * particles.  Errors (BIB_EINVAL) leave the lattice unchanged, except a file that changes while it
 * is being read. ---- */
bib_status bib_checkpoint_save(bib_ctx* ctx, int32_t h, const char* path);
bib_status bib_checkpoint_load(bib_ctx* ctx, int32_t h, const char* path);

/* ---- the reference's own particle files.  `dir` is the folder of the reference's FileName
 * (global::directories() output / input folder; NULL or "" = the working directory); missing
 * folders are created.
 * bib_particles_save_plb / _load_plb: ImmersedBoundaryDynamics3D::save_checkpoint /
 * load_checkpoint (ImmersedBoundaryDynamics_io.hh:17-159).  `name` is taken without folder and
 * extension, as FileName does.  Save writes the text header <dir>/<name>.plb (particle count, file
 * count 1, "<name>/0.plb") and the binary <dir>/<name>/0.plb: an int64 particle count, then each
 * particle's pack (ParticleBase.hh:218-224, DeformableParticle3D.hh:277-287, DeformableCapsule.hh:
 * 217-223, RBCParticle.hh:344-350) with its positions, vertex velocities and vertex forces.
 * Capsules (either shear law) and RBCs only: another model gives BIB_EUNSUPPORTED and no file.
 * Load reads every file the header lists (any rank count), maps each centre of mass to the
 * periodic grid as add_particle does, and replaces the lattice's particles; the ids must be
 * 0 .. n-1 (BIB_EUNSUPPORTED otherwise) and the shapes must be stored under the same ids.
 * bib_particles_write_vtu: write_particles_as_vtk (ImmersedBoundaryDynamics_io.hh:161-176), one
 * file <dir>/obj<id>-<iter>.vtu per particle in ParticleBase3D::write_vtk's layout
 * (ParticleBase.hh:270-390): Float32 positions and vertex forces, Int32 triangles, raw appended data.
 * bib_particle_write_vtu: ParticleBase3D::write_vtk of one particle to `path`.
 * bib_particles_write_lightweight: write_lightweight_particle_data (ImmersedBoundaryDynamics_io.hh:
 * 178-199): <dir>/objsP0-<iter>.txt, "iteration:<iter>" then per particle
 * tag:id:centre:gyration tensor (xx xy xz yy yz zz):volume (DeformableParticle3D.hh:318-333). ---- */
bib_status bib_particles_save_plb(bib_ctx* ctx, int32_t h, const char* dir, const char* name);
bib_status bib_particles_load_plb(bib_ctx* ctx, int32_t h, const char* dir, const char* name);
bib_status bib_particles_write_vtu(bib_ctx* ctx, int32_t h, const char* dir, uint64_t iter);
bib_status bib_particle_write_vtu(bib_ctx* ctx, int32_t h, int32_t pid, const char* path);
bib_status bib_particles_write_lightweight(bib_ctx* ctx, int32_t h, const char* dir, uint64_t iter);
/* parallelIO::save(lattice, name, false) / parallelIO::load(name, lattice, false) (io/multiBlockWriter3D.cpp:
 * 53-137, 201-213; io/multiBlockReader3D.cpp:135-268): the lattice in Palabos' static-content checkpoint,
 * an XML spec <dir>/<name>.plb and the raw cells <dir>/<name>.dat (x-major, z fastest; per cell 19
 * f-bar, the force and the phase as doubles, BIB_LAYOUT_PALABOS_F64).  Save writes one block of
 * descriptor ForcedPhaseD3Q19.  Load reads any block decomposition (a checkpoint of a multi-rank run)
 * of ForcedPhaseD3Q19 or ForcedD3Q19 (then the phase field is kept) into a lattice of the same size,
 * as bib_lattice_send does; dynamic content gives BIB_EUNSUPPORTED. */
bib_status bib_lattice_save_plb(bib_ctx* ctx, int32_t h, const char* dir, const char* name);
bib_status bib_lattice_load_plb(bib_ctx* ctx, int32_t h, const char* dir, const char* name);

/* ---- coupled step: computeVelocity -> setExternalVector -> IB step -> collideAndStream ---- */
bib_status bib_step(bib_ctx* ctx, int32_t h, int64_t nsteps);
/* bib_step bracketed by CUDA events on the context's stream; *ms = device time, synchronises */
bib_status bib_step_timed(bib_ctx* ctx, int32_t h, int64_t nsteps, double* ms);
/* stream the context's work into CUDA-graph replays (1) or plain launches (0) */
bib_status bib_set_graph_mode(bib_ctx* ctx, int32_t enabled);
/* kernel launches in one coupled step of lattice h, counted in the CUDA graph that bib_step
 * replays (its kernel nodes; memset nodes are not counted); BIB_EINVAL before the first
 * graph-replayed bib_step of the lattice.  No reference counterpart (instrumentation). */
bib_status bib_step_kernel_count(bib_ctx* ctx, int32_t h, int32_t* kernels_per_step);
/* scan populations and vertex positions for NaN / Inf: BIB_OK or BIB_ENAN; BIB_ETIMEOUT if a
 * bounded device wait of an earlier step gave up, BIB_EOVERFLOW if an earlier voxelization met a
 * lattice column crossed by more than 64 membrane triangles or a triangle wider than the lattice
 * (each flag is cleared by the call) */
bib_status bib_check_health(bib_ctx* ctx, int32_t h);
/* kernel selection and tile size of the collide-and-stream step (no reference counterpart);
 * BIB_EUNSUPPORTED if BIB_KERNEL_STAGED is forced on a lattice whose x-rows do not fit it */
bib_status bib_lattice_set_tuning(bib_ctx* ctx, int32_t h, const bib_tuning* t);

/* ---- batches: several independent lattices stepped in lockstep, one launch per kernel for all of them,
 * replayed as CUDA graphs (no reference counterpart; the reference runs one domain per process).  The
 * lattices share storage, collision and delta kernel, spread with atomics and fit the staged
 * collide-and-stream kernel.  A batch step is a bib_step of every lattice. ---- */
typedef struct {
    int32_t tile_cells;     /* staged collide-and-stream tile (cells, whole x-rows); 0 = default */
    int32_t stages;         /* its pipeline depth 2..4; 0 = automatic */
    int32_t membrane_block; /* threads per particle of the membrane kernel: 64, 128, 256 or 512 (0 = 256) */
    int32_t reserved[5];
} bib_batch_tuning;
bib_status bib_batch_create(bib_ctx* ctx, const int32_t* handles, int32_t n, int32_t* batch);
bib_status bib_batch_destroy(bib_ctx* ctx, int32_t batch);
bib_status bib_batch_step(bib_ctx* ctx, int32_t batch, int64_t nsteps);
bib_status bib_batch_step_timed(bib_ctx* ctx, int32_t batch, int64_t nsteps, double* ms);
bib_status bib_batch_set_tuning(bib_ctx* ctx, int32_t batch, const bib_batch_tuning* t);
/* Autotuner: times every tile size x stage count, then every membrane block size, each over `steps`
 * real coupled steps (the batch advances by those steps), and keeps the fastest; *chosen may be NULL. */
bib_status bib_batch_autotune(bib_ctx* ctx, int32_t batch, int32_t steps, bib_batch_tuning* chosen);

/* ---- deterministic force spreading that allocates no device memory (no counterpart in the reference) ----
 * For callers that cannot let the library allocate device memory: a host whose pool allocator already
 * holds the GPU's free memory (a cudaMalloc by the library would fail or fragment it), or a stepping loop
 * that cannot take the device-wide synchronisation of cudaMalloc / cudaFree.
 * Adds the delta-weighted forces of nvert vertices into `field`, in the order of BIB_SPREAD_DETERMINISTIC,
 * with the geometry, periodicity, delta kernel and field offset of lattice h.  pos and force are device
 * arrays of nvert x 3 doubles; field is a device array of 3 x nz x ny x nx values (x fastest), double for a
 * BIB_STORAGE_F64 lattice and float otherwise.  The sort scratch is one static device array of the library
 * (BIB_SPREAD_NOALLOC_SCRATCH_BYTES); nvert x support^3 (support 3 for Roma, 4 for Peskin) above
 * BIB_SPREAD_NOALLOC_MAX_ENTRIES is rejected with BIB_EINVAL before any work is queued.
 * bib_create resolves the array's device address on the context's device (the set-up step), so the
 * entry point makes no runtime query of its own; after a cudaDeviceReset, which invalidates every
 * context, create a new context (it resolves the address anew).  Every call uses the same array, so calls
 * that overlap in time on one device (from two contexts, two threads, or streams not ordered with each
 * other) race on it.  The work is queued on the context's stream; the call returns without
 * synchronising. */
#define BIB_SPREAD_NOALLOC_MAX_ENTRIES (1 << 20)
#define BIB_SPREAD_NOALLOC_SCRATCH_BYTES (17u << 20)
bib_status bib_spread_forces_noalloc(bib_ctx* ctx, int32_t h, const double* pos, const double* force, int64_t nvert,
                                     void* field);

/* ---- timing: per-kernel-group device time (ms) of the last bib_step call when profiling is on ---- */
bib_status bib_set_profiling(bib_ctx* ctx, int32_t enabled);
/* out[5] = {membrane forces, spreading, collide+stream, walls, interpolation+move+update};
 * cumulative device milliseconds since profiling was enabled.  The groups are the reference's
 * Profile timers (fsi/Profile.h:26-97): compute_forces, spread_forces, lbm (collideAndStream and,
 * as out[3], its wall processors), interpolate + move; with profiling on, each step also opens
 * NVTX ranges of those names around its phases (steps run eagerly, not as graphs). */
bib_status bib_profile_read(bib_ctx* ctx, double* out, int32_t n);

#ifdef __cplusplus
}
#endif
#endif
