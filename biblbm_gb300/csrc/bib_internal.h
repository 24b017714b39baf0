// Internal declarations of biblbm_gb300: device data layout and kernel launchers.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <array>
#include <string>
#include <vector>

#include "bib/bib.h"

namespace bib {

constexpr int Q = 19;
// Bound of every device-side wait (the staged kernel's mbarrier waits on its own bulk copies)
constexpr uint64_t kDefaultWaitNs = 2000000000ull;

// Lattice geometry and physics parameters as the kernels see them (passed by value).
struct LatticeDesc {
    int nx, ny, nz;
    int64_t n;        // nx*ny*nz
    int64_t stride;   // distance between two population arrays (>= n, padded to 128)
    int px, py, pz;   // periodic flags
    int wall_y, wall_z;
    int fd_walls;     // finite-difference velocity walls on the y = 0 and y = ny-1 planes
    int collision;
    int use_phase;
    int has_types;    // per-cell dynamics (celltype) present
    double omega, omega_inner, trt_magic;
    double omega_c0, omega_c1;  // omega for phase 0 and 1: w0*w1/(c*w0 + (1-c)*w1)
    double inv_n[3];            // 1/nx, 1/ny, 1/nz (Arithmetic1D's Linv, Periodicity.h:73-78)
    double wall_u[4][3];
    double body[3];
    float scale, inv_scale;     // FP16 storage scale
};

struct IbDesc {
    int dirac;
    int spread_mode;
    double offset;
    // ImmersedBoundaryDynamics3D::set_boundary with a PipeBoundary along x: near-wall TopHat
    // blend of interpolation and spreading, wall reflection of the move (has_pipe = 0: none)
    int has_pipe = 0;
    double pipe_y0 = 0.0, pipe_z0 = 0.0, pipe_r = 0.0;
};

// Geometry of one reference shape, device resident.
struct ShapeDev {
    int nv, nt, nl, np;
    double area, volume;  // rest area A0 and volume V0
    double* rest;         // 3*nv
    int* tri;             // 3*nt
    int* tri4;            // 4*nt: the corners of each triangle and a pad, for 16-byte loads
    double* tri_area;     // nt
    int* links;           // 2*nl
    double* link_len;     // nl
    int* pairs;           // 4*np
    double* pair_cs;      // 2*np
    int* inc_off;         // nv+1: per-vertex incidence lists (links, triangles, pairs)
    int* inc;             // (type << 29) | element id
    // FP32 copies for the reduced-precision element kernels
    float* tri_rest_f;    // 4*nt: rest l0, l0', cos(phi0), sin(phi0) of each triangle
    float* tri_area_f;    // nt
    float* pair_cs_f;     // 2*np
};

// One particle as the device kernels see it.
struct ParticleDev {
    int shape, model;
    int v0, nv;           // first vertex in the concatenated vertex arrays, vertex count
    int nt, nl, np;
    const double* rest;
    const int* tri;
    const int* tri4;
    const double* tri_area;
    const int* links;
    const double* link_len;
    const int* pairs;
    const double* pair_cs;
    const int* inc_off;
    const int* inc;
    const float* tri_rest_f;
    const float* tri_area_f;
    const float* pair_cs_f;
    int inst;             // lattice of the particle within a batch (0 for a single lattice)
    int lpid;             // particle index within its lattice
    double A0;
    double prm[BIB_P_COUNT];
};

// Per-particle state kept on the device: {area, volume, com[3]}.
constexpr int STATS = 5;

// A node of the second-order rigid wall (GuoRigidWallBoundary::NodeInfo,
// fsi/GuoBoundaryCondition.h:19-26): the wall node, the population index of its lattice vector
// towards the fluid, 1 - t of the wall crossing, the wall velocity, and whether it carries
// NoDynamics (equilibrium 0).
struct GuoNode {
    int x, y, z;
    int dir;
    int nodyn;
    double delta;
    double u[3];
};

// Interaction potentials and the wall / particle-particle interactions of a lattice.
struct PotentialDev {
    int kind;  // BIB_POTENTIAL_*
    double r0, beta, strength;
};
struct Interactions {
    int nwall = 0;
    int wall_axis[BIB_MAX_WALL_INTERACTIONS] = {};
    double wall_lo[BIB_MAX_WALL_INTERACTIONS] = {}, wall_hi[BIB_MAX_WALL_INTERACTIONS] = {};
    // wall_axis 3: a PipeBoundary along x through (wall_lo, wall_hi) = (y0, z0) of radius wall_r
    double wall_r[BIB_MAX_WALL_INTERACTIONS] = {};
    PotentialDev wall[BIB_MAX_WALL_INTERACTIONS] = {};
    int npp = 0;
    PotentialDev pp[BIB_MAX_PP_INTERACTIONS] = {};
    double pp_cut = 0.0;  // largest particle-particle cutoff
    int pp_search = 0;    // BIB_PAIR_SEARCH_*
};

// Hashed cell list of the pair search: cells of at least the cutoff (nc per axis, size cs),
// hashed into `table` buckets; vertices sorted by bucket, [start, end) per bucket.
struct PairGrid {
    int nc[3] = {1, 1, 1};
    double cs[3] = {1.0, 1.0, 1.0};
    unsigned table = 0;  // power of two
    int bits = 0;
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* ids[2] = {nullptr, nullptr};
    int* start = nullptr;
    int* end = nullptr;
    void* temp = nullptr;
    size_t temp_bytes = 0;
};

// The reference's collision grid (fsi/Grid.hh over the box [lo - 1/2, hi + 1/2 - eps] per axis,
// one envelope layer; CollisionForces.h): nc cells per axis of size cs, cell 0 at g0; vertices
// strictly inside (lo_, hi_) (the box enlarged by the cutoff) are keyed by their cell.
struct RefGrid {
    int nc[3];
    int per[3];
    int ncell;
    int nvert;
    double cs[3], g0[3], b0[3];
    double lo[3], hi[3];
    double L[3], Linv[3];  // periodic arithmetic of the box
};
struct RefGridBuffers {
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* ids[2] = {nullptr, nullptr};
    int* start = nullptr;  // ncell + 1 entries each, zero between uses
    int* end = nullptr;
    float4* posf = nullptr;  // the vertex positions rounded to FP32 (the pair pre-test)
    void* temp = nullptr;
    size_t temp_bytes = 0;
    int bits = 0;
};
int64_t ref_grid_cells(const int64_t* box);  // cells of the grid over box (envelope included)
constexpr int64_t kMaxRefGridCells = (int64_t)1 << 30;
RefGrid ref_grid(const int64_t* box, const int* periodic, double cut, int nvert);
int ref_grid_bits(int64_t ncell);
size_t ref_grid_temp_bytes(int nvert, int bits);
// forces of one potential by the reference's grid search; zero: start from zero forces (and
// write the vertices outside the grid), else add in place; wall {y0, z0, radius} or null: the
// growth stage's pipe wall pass
void launch_ref_grid_forces(const RefGrid& g, const RefGridBuffers& B, const PotentialDev& pot, const double* pos,
                            const int* owner, double* force, bool zero, const double* wall, cudaStream_t s);

// Rigid copies of shapes in the growth stage of the initial distribution (device pointers).
struct GrowthView {
    int np = 0;
    const int* shape = nullptr;     // per particle
    const int* part_v0 = nullptr;   // first vertex of each particle
    const int* shape_nv = nullptr;  // per shape
    const int* shape_v0 = nullptr;  // first vertex of each shape in verts
    const double* verts = nullptr;  // the shapes' vertices
    const double* volume = nullptr; // per shape
    const double* inertia = nullptr;  // 9 per shape, about the origin
    double* com = nullptr;
    double* quat = nullptr;
    double* vel = nullptr;
    double* omega = nullptr;
    double* pos = nullptr;
    const double* force = nullptr;
    double* torque = nullptr;  // 3 per vertex, scratch
    double density = 1.0, damping = 0.0;
    long long* it = nullptr;          // the iteration counter
    const double* scales = nullptr;   // the scale of iteration k * every
    long long every = 1;
    double* scale_now = nullptr;      // the current scale
    int per[3] = {0, 0, 0};
    double x0[3] = {0, 0, 0}, L[3] = {1, 1, 1}, Linv[3] = {1, 1, 1};
};
void launch_rigid_nodes(const GrowthView& G, double scale, cudaStream_t s);
void launch_rigid_rescale(const GrowthView& G, cudaStream_t s);  // at the iteration *G.it
void launch_rigid_move(const GrowthView& G, cudaStream_t s);     // advances *G.it

// What the immersed-boundary kernels need of one lattice for one step (buffer parities
// resolved).  A single lattice passes one view by value; a batch passes a device table of
// views, indexed per vertex (through the vertex -> lattice map) or per particle (inst).
struct IbView {
    LatticeDesc d;
    IbDesc ib;
    const double* pos;   // X_n
    double* pos_next;    // X_{n+1}
    const void* u;       // velocity field, 4 values per cell (FP64 / FP32 / FP16 as the populations)
    double* vel;
    double* force;       // vertex forces
    void* F;             // spreading target (field type as u)
    double* stats;       // STATS per particle
    int vbase;           // batch numbering of the lattice's first vertex
    int nvert;
    Interactions inter;  // wall interactions are applied by the membrane kernel
    // sparse force reset (single lattices, FP32 fields): the spreading records the first
    // support node of every vertex (x, y, z, 1; w = 0 outside the envelope) in spread_lo, and
    // the interpolation adds (Fold - body) / 2 of the force field of the previous step to the
    // velocity field j / rho + body / 2 that the collision wrote.  Null: not used.
    int4* spread_lo = nullptr;
    const void* Fold = nullptr;
    const int* order = nullptr;  // single lattices: the vertex each interpolation thread takes
};

// Per-launch constants of the collision in the compute type C.
template <class C>
struct CollideParams {
    C om0, om1;      // relaxation frequency of phase 0 / 1 (BGK + Guo) or the omega of BGK / TRT
    C omm;           // TRT: omega of the antisymmetric part
    C S, invS;       // storage scale (FP16) and its inverse, 1 otherwise
    C body[3];       // body force, the reset value of the previous force field
    C wall_u[2][3];  // velocity of the finite-difference wall rows y = 0, ny - 1
    C mw[4][19];     // moving-wall bounce-back term per wall face and population, storage units
};

// One lattice of a batched collide-and-stream step (buffer parities resolved): the staged
// kernel maps its global tile index to (lattice, local tile) through tile0.
struct CollideView {
    LatticeDesc d;
    const void* fin;
    void* fout;
    const void* wall;
    const void* Fcol;       // spread force of this step
    void* Fprev;            // force of the incoming state (reset to the body force)
    void* u;                // velocity output
    const uint8_t* phase;
    const uint8_t* celltype;
    int64_t tile0;          // first global tile of this lattice
    int64_t ntiles;
    int R, Ct, tiles_y;     // rows per tile, cells per tile, tiles per z-plane
    unsigned tx_bytes;      // bytes copied in per tile
    alignas(16) unsigned char cp[sizeof(CollideParams<double>)];  // CollideParams<compute type>
};

struct ShapeHost {
    std::vector<double> rest, tri_area, link_len, pair_cs;
    std::vector<int> tri, tri4, links, pairs, inc_off, inc;
    std::vector<int> order;  // vertices in a spatially clustered order (Morton order of the rest shape)
    std::vector<float> tri_rest_f, tri_area_f, pair_cs_f;
    double area = 0, volume = 0;
    std::string tag;  // ParticleShape tag (ParticleShape.h:64), the shape's name in text output
    ShapeDev dev{};
};

struct ParticleHost {
    int shape, model;
    int v0, nv;
    std::vector<double> prm;
};

// Device state of one lattice.
//
// Populations use a pull scheme: buffer f[cur] holds the post-collision populations of
// the previous step, f*(x), so the post-streaming state the reference keeps between
// steps is f_i(x) = f*_i(x - c_i) (with bounce-back / wall rules at the faces).  The
// collide-and-stream kernel gathers f_i(x), emits the velocity field
// u = j/rho + F_prev/2 the reference's computeVelocity would produce for this state,
// collides with the force spread in this step and writes f*(x) into f[1-cur].  Nodes on
// finite-difference velocity walls read their populations from wall[] instead, which the
// wall kernel fills after every collide-and-stream.
//
// Forces are double-buffered: F[fe] holds the external force of the current state (the
// reference's Cell externals), F[1-fe] is the target of the spreading of the next step.
struct Lattice {
    LatticeDesc d{};
    IbDesc ib{0, 0, -1.0};
    int storage = BIB_STORAGE_F64;
    void* f[2] = {nullptr, nullptr};
    int cur = 0;
    void* wall = nullptr;             // 2 sides x nx x nz x 19 populations of FD wall nodes
    void* F[2] = {nullptr, nullptr};  // force fields (double for F64 storage, float otherwise)
    int fe = 0;
    bool target_clean = false;        // F[1-fe] holds the body force, ready to receive spreading
    // Sparse force reset (opt-in; reduced-precision storage, coupled step, no phase field, cell
    // types or pipe boundary): the collision reads only the spread force of its step, and the field of
    // the previous step is reset to the body force only where its spreading wrote (the support
    // nodes recorded in spread_lo[b] for F[b]).  sparse_ok[b]: F[b] differs from the body force
    // only at the nodes in spread_lo[b].
    int4* spread_lo[2] = {nullptr, nullptr};
    bool sparse_ok[2] = {false, false};
    bool sparse_reset = false;  // tuning: the sparse reset where the lattice allows it
    uint64_t wait_ns = kDefaultWaitNs;  // bound of the staged kernel's hand-off waits
    int64_t withhold_tile = -1;         // failure testing: a staged tile whose copies are not issued
    void* u = nullptr;                // velocity field, (ux, uy, uz, 0) per cell (double for F64 storage, float otherwise)
    uint8_t* phase = nullptr;
    uint8_t* celltype = nullptr;      // BIB_CELL_* per cell, or nullptr: every cell has the lattice's dynamics
    GuoNode* guo = nullptr;           // second-order rigid-wall nodes, rebuilt after every collide-and-stream
    int nguo = 0;
    // immersed boundary
    std::vector<ParticleHost> parts;
    int nvert = 0;
    double* pos[2] = {nullptr, nullptr};  // vertex positions, swapped every step
    int pcur = 0;
    double* vel = nullptr;
    double* force = nullptr;
    double* stats = nullptr;              // STATS per particle
    ParticleDev* pdev = nullptr;
    std::vector<ParticleDev> pdev_host;  // host copy of pdev (batch tables are built from it)
    int* vert_particle = nullptr;         // global vertex -> particle
    int* visit_order = nullptr;          // the interpolation's visiting order of the vertices
    Interactions inter;                   // wall and particle-particle interactions
    PairGrid pgrid;                       // pair search of the particle-particle interactions
    RefGridBuffers rgrid;                 // ... when they use the reference's collision grid
    int max_nv = 0;
    int max_elems = 0;            // most triangles, links or pairs of one particle
    int max_nt = 0;               // most triangles of one particle
    double* upd_partial = nullptr;  // partial sums of the split update (particles x 64 x 5)
    bool particles_dirty = true;  // host copies below are authoritative until uploaded
    std::vector<double> host_pos;    // concatenated vertex positions
    std::vector<double> host_stats;  // STATS per particle
    size_t membrane_smem = 0;
    // deterministic spreading: (target cell, entry) pairs and their radix-sorted copies
    uint32_t* sort_keys[2] = {nullptr, nullptr};
    uint32_t* sort_ids[2] = {nullptr, nullptr};
    void* sort_temp = nullptr;
    size_t sort_temp_bytes = 0;
    // collide-and-stream kernel selection (BIB_KERNEL_*), staged tile size (0 = default)
    int collide_kernel = BIB_KERNEL_AUTO;
    int tile_cells = 0;
    int stages = 0;           // staged kernel pipeline depth (0 = automatic)
    int membrane_block = 256; // threads per particle of the membrane kernel
    int* wait_err = nullptr;  // device word set by a bounded device wait that gave up
    // voxelization of the membranes into the phase field (lattices with a phase field and particles)
    int* vox_count = nullptr;  // crossings per (x, y) column, zero between launches
    double* vox_z = nullptr;   // kVoxelCap heights per column, slot-major
    int* vox_err = nullptr;    // device word set when a column held more than kVoxelCap crossings
    uint64_t version = 0;     // bumped whenever the particle buffers are (re)allocated
    uint64_t iteration = 0;   // steps taken (coupled, IB-only and collide-and-stream), kept in checkpoints
    int handle = -1;
};

// ---- kernel launchers (lattice_kernels.cu) ----
// How a collide-and-stream treats the force fields and the velocity field.
enum class Coupling {
    kNone,    // collision with F[fe], no side outputs
    kDense,   // velocity j/rho + F[fe]/2 written, collision with F[1-fe], F[fe] reset to the body force
    kSparse,  // velocity j/rho + body/2 written, collision with F[1-fe]; F[fe] left for the sparse reset
};
void launch_collide_stream(const Lattice& L, Coupling mode, cudaStream_t s);
// shared-memory staged variant (collide_staged.cu); false if the lattice shape does not fit it
bool launch_collide_stream_staged(const Lattice& L, Coupling mode, cudaStream_t s);
bool collide_staged_fits(const Lattice& L);  // both step kinds fit the staged kernel
void launch_fd_walls(const Lattice& L, int buf, int fbuf, cudaStream_t s);
void launch_velocity_field(const Lattice& L, cudaStream_t s);  // u from the current state and F[fe]
void launch_velocity_export(const Lattice& L, double* u, cudaStream_t s);
void launch_init_equilibrium(const Lattice& L, const double* rho, const double* u, cudaStream_t s);
// populations of planes z0 .. z0 + nzc - 1 from / to FP64 SoA slices of `pitch` cells
void launch_import_planes(const Lattice& L, const double* src, int z0, int nzc, int64_t pitch, cudaStream_t s);
void launch_export_planes(const Lattice& L, double* dst, int z0, int nzc, int64_t pitch, cudaStream_t s);
// cells w0 .. w0 + count - 1 of the cell-major wire order (x slowest, z fastest), `per` doubles
// per cell: 19 populations (CoProcessor3D) or 19 populations, the force and the phase (Palabos
// static content; the force goes to / comes from F[fe])
void launch_import_aos(const Lattice& L, const double* src, int per, int64_t w0, int64_t count, cudaStream_t s);
void launch_export_aos(const Lattice& L, double* dst, int per, int64_t w0, int64_t count, cudaStream_t s);
void launch_force_import(const Lattice& L, int buf, const double* src, cudaStream_t s);
void launch_force_export(const Lattice& L, int buf, double* dst, cudaStream_t s);
void launch_force_fill(const Lattice& L, int buf, cudaStream_t s);
void launch_phase_import(const Lattice& L, const double* src, cudaStream_t s);
void launch_nan_scan(const Lattice& L, int* flag, cudaStream_t s);
// dst[i] = src[i] for i < n (dst may be page-locked host memory mapped for the device)
void launch_copy_f64(double* dst, const double* src, size_t n, cudaStream_t s);

// ---- kernel launchers (ib_kernels.cu) ----
void launch_membrane_forces(const Lattice& L, cudaStream_t s);
// spreading into F[fbuf]; with `record` the support nodes go to spread_lo[fbuf]
void launch_spread(const Lattice& L, int fbuf, cudaStream_t s, bool record = false);
// vel and pos[1-pcur] = pos + vel; fold >= 0: the velocity field is the sparse-reset form and
// (F[fold] - body) / 2 is added to it at the support nodes
void launch_interpolate_move(const Lattice& L, cudaStream_t s, int fold = -1);
// F[fbuf] := body force at the support nodes in spread_lo[fbuf]
void launch_force_clear(const Lattice& L, int fbuf, cudaStream_t s);
void launch_particle_update(const Lattice& L, cudaStream_t s);   // area/volume/COM of pos[1-pcur] + remap
// particle-particle interaction forces at pos[pcur] added to the vertex forces (no-op without)
void launch_pp_forces(const Lattice& L, cudaStream_t s);
size_t pp_sort_temp_bytes(int nvert, int bits);
// one relax_nodes iteration of the shape calibration of the single RBC of L (pos[pcur] -> pos[1-pcur])
void launch_rbc_relax(const Lattice& L, double damping, long long* iter, long long n_it, double vol_start,
                      double vol_final, cudaStream_t s);
constexpr int kVoxelCap = 64;  // membrane crossings one (x, y) column can hold
void launch_voxelize(const Lattice& L, const double* pos, cudaStream_t s);  // phase field of the membranes at pos
size_t membrane_smem_bytes(int max_nv);
size_t spread_sort_temp_bytes(int64_t nentries);
void configure_membrane_kernel(size_t smem);
// Deterministic spreading into a field of stride d.stride with caller-provided scratch:
// (cell, entry) keys and entry ids, two buffers each of nvert * support^3 words, and the
// radix sort's temporary storage (spread_sort_temp_bytes_pingpong bytes).
size_t spread_sort_temp_bytes_pingpong(int64_t nentries, int end_bit);
cudaError_t launch_spread_sorted(const LatticeDesc& d, const IbDesc& ib, bool f64_field, int nvert, const double* pos,
                                 const double* force, void* field, uint32_t* keys0, uint32_t* keys1, uint32_t* ids0,
                                 uint32_t* ids1, void* temp, size_t temp_bytes, cudaStream_t s);
int spread_key_bits(int64_t n);

// ---- batched steps: one launch per kernel for all lattices of a batch ----
// Device tables of one step parity (the lattices of a batch advance in lockstep).
struct BatchLaunch {
    int n = 0;                          // lattices
    int storage = 0, collision = 0, dirac = 0;
    const IbView* views = nullptr;      // n views of this step (spreading target = F[1-fe])
    const CollideView* cviews = nullptr;  // n collide views of this step
    const CollideView* wviews = nullptr;  // n collide views of the next state (finite-difference walls)
    const ParticleDev* parts = nullptr; // all particles, ParticleDev::inst = lattice
    int nparts = 0;
    const int* vinst = nullptr;         // batch vertex -> lattice
    int nvert = 0;
    int max_nv = 0;
    size_t membrane_smem = 0;
    int64_t ntiles = 0;                 // staged tiles over all lattices
    int stages = 0;                     // staged pipeline depth (0 = automatic)
    int any_fd = 0;                     // some lattice has finite-difference walls
    int nx_max = 0, nz_max = 0;
    int* wait_err = nullptr;            // device word of the bounded waits
};
IbView single_view(const Lattice& L, int fbuf);  // parities of L; fbuf < 0: no spreading target
void launch_membrane_batch(const BatchLaunch& B, int block, cudaStream_t s);
void launch_spread_batch(const BatchLaunch& B, cudaStream_t s);
void launch_interpolate_batch(const BatchLaunch& B, cudaStream_t s);
void launch_update_batch(const BatchLaunch& B, cudaStream_t s);
// staged collide-and-stream over the tiles of all lattices (coupled step); false if a lattice
// does not fit the staged kernel
bool launch_collide_batch(const BatchLaunch& B, cudaStream_t s);
bool collide_batch_fits(int storage, int collision, int stages);  // shared memory of that many stages
void launch_fd_walls_batch(const BatchLaunch& B, cudaStream_t s);
// fills the tile geometry and collision constants of a collide view; false if L does not fit
bool staged_collide_view(const Lattice& L, int tile_cells, CollideView& v);

// ---- spreading without device allocation (noalloc.cu) ----
// device address of the scratch array on the current device (called by bib_create)
bib_status spread_scratch_address(void** out, std::string& msg);
bib_status spread_noalloc(const Lattice& L, int device, void* scratch, cudaStream_t s, const double* pos, const double* force,
                          int64_t nvert, void* field, std::string& msg);

// ---- the reference's particle file formats (reference_files.cu) ----
// Particle type ids of the reference's particle factory (ParticleFactory.hh:63-66): registration
// order of the particle classes in a program that includes fsi/headers.hh
constexpr int64_t kPlbTypeCapsule = 0;  // DeformableCapsuleParticle, DeformableCapsule.hh:43
constexpr int64_t kPlbTypeRbc = 1;      // RBCParticle, RBCParticle.hh:123
struct PlbParticle {
    int64_t shape = 0, id = 0;
    int model = 0;  // BIB_MODEL_*
    bool voxelize = true;
    std::vector<double> pos, vel, force;  // 3 per vertex
    double prm[BIB_P_COUNT] = {};
};
// append one particle's pack; false (err set) for a model without a reference particle type
bool plb_pack(std::string& out, const PlbParticle& p, std::string& err);
// read one particle's pack at it (advanced past it); shape_nv: vertex count per shape id
bool plb_unpack(const char*& it, const char* end, const std::vector<int>& shape_nv, PlbParticle& p,
                std::string& err);
std::string vtu_bytes(const double* pos, const double* force, int nv, const int* tri, int nt);
std::string lightweight_line(const std::string& tag, int64_t id, const double* pos, int nv, const double* com,
                             double volume);
bool mkdir_p(const std::string& dir);
// parallelIO XML spec of a one-block ForcedPhaseD3Q19 lattice with static content of `bytes` bytes
std::string plb_lattice_xml(const std::string& dat_file, int nx, int ny, int nz, bool vof, int64_t bytes);
struct PlbLatticeSpec {
    int cell_dim = 0;
    bool dynamic = false;
    std::string datatype, file, ordering;
    int64_t box[6] = {};                      // x0 x1 y0 y1 z0 z1, inclusive
    std::vector<std::array<int64_t, 6>> comps;  // block boxes
    std::vector<int64_t> offsets;             // end offset of each block's bytes
};
bool plb_lattice_parse(const std::string& xml, PlbLatticeSpec& s, std::string& err);

}  // namespace bib
