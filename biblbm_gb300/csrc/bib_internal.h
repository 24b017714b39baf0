// Internal declarations of biblbm_gb300: device data layout and kernel launchers.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "bib/bib.h"

namespace bib {

constexpr int Q = 19;

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
};

// Geometry of one reference shape, device resident.
struct ShapeDev {
    int nv, nt, nl, np;
    double area, volume;  // rest area A0 and volume V0
    double* rest;         // 3*nv
    int* tri;             // 3*nt
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
    double A0;
    double prm[BIB_P_COUNT];
};

// Per-particle state kept on the device: {area, volume, com[3]}.
constexpr int STATS = 5;

struct ShapeHost {
    std::vector<double> rest, tri_area, link_len, pair_cs;
    std::vector<int> tri, links, pairs, inc_off, inc;
    std::vector<float> tri_rest_f, tri_area_f, pair_cs_f;
    double area = 0, volume = 0;
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
    void* u = nullptr;                // velocity field (double for F64 storage, float otherwise)
    uint8_t* phase = nullptr;
    // immersed boundary
    std::vector<ParticleHost> parts;
    int nvert = 0;
    double* pos[2] = {nullptr, nullptr};  // vertex positions, swapped every step
    int pcur = 0;
    double* vel = nullptr;
    double* force = nullptr;
    double* stats = nullptr;              // STATS per particle
    ParticleDev* pdev = nullptr;
    int* vert_particle = nullptr;         // global vertex -> particle
    int max_nv = 0;
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
    int* wait_err = nullptr;  // device word set by a bounded device wait that gave up
    int handle = -1;
};

// ---- kernel launchers (lattice_kernels.cu) ----
// coupled = true: velocity output, collision with the spread force F[1-fe], F[fe] reset
// to the body force afterwards.  coupled = false: collision with F[fe], no side outputs.
void launch_collide_stream(const Lattice& L, bool coupled, cudaStream_t s);
// shared-memory staged variant (collide_staged.cu); false if the lattice shape does not fit it
bool launch_collide_stream_staged(const Lattice& L, bool coupled, cudaStream_t s);
bool collide_staged_fits(const Lattice& L);  // both step kinds fit the staged kernel
void launch_fd_walls(const Lattice& L, int buf, int fbuf, cudaStream_t s);
void launch_velocity_field(const Lattice& L, cudaStream_t s);  // u from the current state and F[fe]
void launch_velocity_export(const Lattice& L, double* u, cudaStream_t s);
void launch_init_equilibrium(const Lattice& L, const double* rho, const double* u, cudaStream_t s);
// populations of planes z0 .. z0 + nzc - 1 from / to FP64 SoA slices of `pitch` cells
void launch_import_planes(const Lattice& L, const double* src, int z0, int nzc, int64_t pitch, cudaStream_t s);
void launch_export_planes(const Lattice& L, double* dst, int z0, int nzc, int64_t pitch, cudaStream_t s);
void launch_force_import(const Lattice& L, int buf, const double* src, cudaStream_t s);
void launch_force_export(const Lattice& L, int buf, double* dst, cudaStream_t s);
void launch_force_fill(const Lattice& L, int buf, cudaStream_t s);
void launch_phase_import(const Lattice& L, const double* src, cudaStream_t s);
void launch_nan_scan(const Lattice& L, int* flag, cudaStream_t s);

// ---- kernel launchers (ib_kernels.cu) ----
void launch_membrane_forces(const Lattice& L, cudaStream_t s);
void launch_spread(const Lattice& L, int fbuf, cudaStream_t s);
void launch_interpolate_move(const Lattice& L, cudaStream_t s);  // vel and pos[1-pcur] = pos + vel
void launch_particle_update(const Lattice& L, cudaStream_t s);   // area/volume/COM of pos[1-pcur] + remap
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

// ---- spreading without device allocation (noalloc.cu) ----
bib_status spread_noalloc(const Lattice& L, int device, cudaStream_t s, const double* pos, const double* force,
                          int64_t nvert, void* field, std::string& msg);

}  // namespace bib
