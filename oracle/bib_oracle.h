/*
 * bib_oracle -- CPU restatement of the reference's hot IB-LBM time step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py load this library; the product never links it.
 *
 * It restates, in plain C and FP64, the arithmetic of niclasberg/biblbm
 * (Palabos + src/fsi) on the hot path, function by function, citing the
 * reference file:line each one follows.  It is pinned against the reference's own
 * code through the fixtures in tests/golden/ (generated by running the compiled
 * reference, see tests/golden/make_golden.py).  Parts with no reference
 * counterpart (TRT collision, halfway / moving-wall bounce-back, the Peskin kernel
 * inside the IB step) are restatements of the published methods and are pinned by
 * analytic solutions in the tests instead.
 *
 * Conventions: lattice fields are structure-of-arrays, component-major, x fastest:
 * value(c, x, y, z) = a[c*n + x + nx*(y + ny*z)], n = nx*ny*nz.  Populations are
 * stored as f-bar = f - t_i (Palabos DefaultRoundOffPolicy, roundOffPolicy.h:72-90)
 * and represent the post-streaming state, the state Palabos holds between steps.
 */
#ifndef BIB_ORACLE_H
#define BIB_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_COLLISION_BGK_GUO_VOF = 0, ORC_COLLISION_BGK = 1, ORC_COLLISION_TRT = 2 };
enum { ORC_WALL_NONE = 0, ORC_WALL_FD_VELOCITY = 1, ORC_WALL_HALFWAY_BB = 2 };
enum { ORC_DIRAC_ROMA = 0, ORC_DIRAC_PESKIN = 1, ORC_DIRAC_TOPHAT = 2 };
enum {
    ORC_MODEL_CAPSULE_NEOHOOKEAN = 0,
    ORC_MODEL_CAPSULE_SKALAK = 1,
    ORC_MODEL_RBC_WLCPOW = 2,
    ORC_MODEL_SKALAK_BENDING = 3
};

/* Index of the membrane parameter vector (12 doubles). */
enum {
    ORC_P_G = 0, ORC_P_C, ORC_P_NU_S, ORC_P_KB, ORC_P_SHEAR_MODULUS, ORC_P_L0, ORC_P_K_AREA_GLOBAL,
    ORC_P_K_AREA_LOCAL, ORC_P_K_VOLUME, ORC_P_VOL_DESIRED, ORC_P_K_BEND, ORC_P_THETA0, ORC_P_COUNT
};

/* a node of GuoRigidWallBoundary (fsi/GuoBoundaryCondition.h:19-26) */
typedef struct {
    int64_t x, y, z;  /* the wall node (outside the boundary) */
    int32_t dir;      /* population index of the lattice vector towards the fluid */
    int32_t nodyn;    /* the node carries NoDynamics: its equilibrium is 0 */
    double delta;     /* 1 - t of the boundary crossing along that vector */
    double u[3];      /* wall velocity */
} orc_guo_node;

typedef struct {
    int64_t nx, ny, nz;
    int32_t periodic[3];
    int32_t collision;
    int32_t wall_y, wall_z;     /* walls on the y / z faces when that axis is not periodic */
    double omega, omega_inner;  /* GuoExternalForceVOFDynamics(omega1, omega2) */
    double trt_magic;
    double wall_u[4][3];        /* velocity of the y-, y+, z-, z+ walls */
    int32_t envelope_swap;      /* reproduce the reference's periodic-envelope omega swap (see .c) */
    const uint8_t* celltype;    /* NULL or per cell: 0 the lattice's dynamics, 1 BounceBack, 2 NoDynamics */
    const orc_guo_node* guo;    /* second-order rigid-wall nodes, rebuilt after every collide-and-stream */
    int64_t nguo;
} orc_lattice;

enum { ORC_CELL_FLUID = 0, ORC_CELL_BOUNCE_BACK = 1, ORC_CELL_NO_DYNAMICS = 2 };

/* ---- voxelization: phase 1 inside the closed membranes, 0 outside ---- */
/* pos: nvt x 3 vertex positions of all particles; tri: ntt x 3 global vertex indices; phase: n cells,
 * updated in place (cells the reference's fill does not reach keep their value). */
void orc_voxelize(const orc_lattice* L, int64_t nvt, const double* pos, int64_t ntt, const int64_t* tri, double* phase);

/* ---- lattice ---- */
void orc_collide_cell(const orc_lattice* L, double* f19, const double* F3, double phase);
void orc_collide_stream(const orc_lattice* L, double* f, double* ftmp, const double* F, const double* phase);
void orc_apply_fd_walls(const orc_lattice* L, double* f, const double* F);
void orc_compute_velocity(const orc_lattice* L, const double* f, const double* F, double* u);
void orc_init_equilibrium(const orc_lattice* L, double* f, const double* rho, const double* u);

/* ---- shapes and membranes ---- */
int64_t orc_shape_connectivity(int64_t nv, const double* xyz, int64_t nt, const int64_t* tri,
                               int64_t* links, double* link_len, int64_t* pairs, double* pair_cs,
                               double* tri_area, double* props, int64_t* npairs);
void orc_particle_update(int64_t nv, const double* pos, int64_t nt, const int64_t* tri, double* out5);
void orc_inertia(const double* pos, int64_t nt, const int64_t* tri, double* out9);
void orc_membrane_forces(int32_t model, const double* prm, int64_t nv, const double* rest, int64_t nt,
                         const int64_t* tri, const double* tri_area, double A0, int64_t nl, const int64_t* links,
                         const double* link_len, int64_t np, const int64_t* pairs, const double* pair_cs,
                         const double* pos, double area, double volume, double* force);

double orc_rbc_shrink_volume(const double* prm_in, int64_t nv, const double* rest, int64_t nt, const int64_t* tri,
                             const double* tri_area, double A0, double V0, int64_t nl, const int64_t* links,
                             const double* link_len, int64_t np, const int64_t* pairs, const double* pair_cs,
                             double vol_final, int64_t n_it, double damping, double* pos, double* vel_out);

/* ---- immersed boundary ---- */
double orc_dirac(int32_t dirac, double r);
void orc_classify(const orc_lattice* L, int32_t dirac, int64_t n, const double* pos, int32_t* cls);
void orc_interpolate(const orc_lattice* L, int32_t dirac, double offset, const double* u, int64_t n,
                     const double* pos, const int32_t* cls, double* vel);
void orc_spread(const orc_lattice* L, int32_t dirac, double offset, int64_t n, const double* pos,
                const double* force, const int32_t* cls, double* F);

/* number of OpenMP threads the lattice loops use (1 without OpenMP) */
int32_t orc_threads(void);

/* ---- coupled system (mirrors the product's C ABI) ---- */
/* BounceBack / NoDynamics cells of the reference's first-order pipe walls (pipe along x) */
void orc_pipe_celltypes(int64_t nx, int64_t ny, int64_t nz, double y0, double z0, double radius, uint8_t* types);
/* the second-order pipe walls: GuoRigidWallBoundary nodes (returns their count; `nodes` may be NULL to
 * count) and the NoDynamics cells beyond radius + 1 (types, 0 elsewhere) */
int64_t orc_pipe_guo_nodes(int64_t nx, int64_t ny, int64_t nz, double y0, double z0, double radius,
                           orc_guo_node* nodes, uint8_t* types);
/* GuoRigidWallBoundaryFunctional::process on a post-streaming state */
void orc_apply_guo(const orc_lattice* L, double* f);

/* interaction potentials (fsi/Potentials.h): kind, cutoff r0 (Morse r_min / spring min_dist), Morse beta, strength */
enum { ORC_POTENTIAL_NONE = 0, ORC_POTENTIAL_MORSE = 1, ORC_POTENTIAL_SPRING = 2 };
typedef struct {
    int32_t kind;
    double r0, beta, strength;
} orc_potential;
double orc_potential_eval(const orc_potential* p, double d);
void orc_wall_forces(const orc_potential* p, int32_t axis, double lo, double hi, int64_t nv, const double* pos,
                     double* force);
void orc_pp_forces_grid(const orc_lattice* L, const orc_potential* p, int64_t nv, const double* pos,
                        const int32_t* owner, double* force);
void orc_pp_forces(const orc_lattice* L, const orc_potential* p, int64_t nv, const double* pos, const int32_t* owner,
                   double* force);

/* growth of the initial distribution (progs/common/create_particles.h:105-161), see the .c */
typedef struct {
    int64_t box[6];            /* x0, x1, y0, y1, z0, z1: the lattice's bounding box */
    int32_t periodic[3];
    int32_t has_wall;
    double wall[3];            /* PipeBoundary y0, z0, radius the collisions keep the vertices inside */
    double min_dist, strength; /* SpringPotential(min_dist, strength), fsi/Potentials.h:58-71 */
    double initial_scale, density, damping;
    int64_t n_it;              /* the scale reaches 1 at iteration n_it */
    int64_t rescale_every;
    int64_t it_end;            /* iterations 0 .. it_end - 1 are run (n_it + 1: the whole growth) */
} orc_growth;
void orc_shape_mass_props(int64_t nt, const int64_t* tri, const double* xyz, double* volume, double* inertia9);
int32_t orc_grow_particles(const orc_growth* g, int32_t nshape, const int64_t* nv, const double* verts,
                           const int64_t* nt, const int64_t* tri, int32_t np, const int32_t* shape, double* com,
                           double* quat, double* pos_out, double* force_out);

typedef struct orc_sys orc_sys;
orc_sys* orc_sys_create(const orc_lattice* L, int32_t dirac, double ib_offset);
void orc_sys_destroy(orc_sys* s);
double* orc_sys_f(orc_sys* s);
double* orc_sys_force(orc_sys* s);
double* orc_sys_phase(orc_sys* s);
void orc_sys_set_body_force(orc_sys* s, const double* b3);
int32_t orc_sys_add_shape(orc_sys* s, int64_t nv, const double* xyz, int64_t nt, const int64_t* tri);
int32_t orc_sys_add_particle(orc_sys* s, int32_t shape, int32_t model, const double* prm, const double* pos);
void orc_sys_init(orc_sys* s);
void orc_sys_step(orc_sys* s, int64_t nsteps);
void orc_sys_set_voxelize(orc_sys* s, int32_t on);  /* revoxelize after every move (and at init) */
/* add_force_decorator(WallInteraction(ParallelPlatesBoundary(lo, hi) normal to `axis`, p)) */
int32_t orc_sys_add_pipe_wall_interaction(orc_sys* s, const orc_potential* p, double y0, double z0, double radius);
int32_t orc_sys_add_wall_interaction(orc_sys* s, const orc_potential* p, int32_t axis, double lo, double hi);
/* add_pp_force(PPPotentialForce(p)); grid = 1 evaluates it with the reference's grid search */
int32_t orc_sys_add_pp_interaction(orc_sys* s, const orc_potential* p, int32_t grid);
/* ImmersedBoundaryDynamics3D::set_boundary with a PipeBoundary along x through (y0, z0): near-wall
 * TopHat blending of interpolation and spreading, wall reflection of the move */
void orc_sys_set_pipe(orc_sys* s, double y0, double z0, double radius);
/* move_vertices: pos += vel, reflected at a pipe wall when pipe = {y0, z0, radius} is given */
void orc_move_vertices(int64_t nv, double* pos, const double* vel, const double* pipe);
void orc_sys_lattice_only_step(orc_sys* s, int64_t nsteps);
void orc_sys_get_particle(orc_sys* s, int32_t pid, double* pos, double* vel, double* force, double* stats5);
void orc_sys_velocity(orc_sys* s, double* u);

#ifdef __cplusplus
}
#endif
#endif
