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
    int64_t stride;   // distance between two population arrays (>= n, padded)
    int px, py, pz;   // periodic flags
    int wall_y, wall_z;
    int collision;
    int use_phase;
    double omega, omega_inner, trt_magic;
    double omega_c0, omega_c1;  // omega for phase 0 and 1: w0*w1/(c*w0 + (1-c)*w1)
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
    double A0;
    double prm[BIB_P_COUNT];
};

// Per-particle state written by the membrane kernel: {area, volume, com[3]}.
constexpr int STATS = 5;

struct ShapeHost {
    std::vector<double> rest, tri_area, link_len, pair_cs;
    std::vector<int> tri, links, pairs;
    double area = 0, volume = 0;
    ShapeDev dev{};
};

struct ParticleHost {
    int shape, model;
    int v0, nv;
    std::vector<double> prm;
};

struct Lattice {
    LatticeDesc d{};
    IbDesc ib{0, 0, -1.0};
    int storage = BIB_STORAGE_F64;
    void* f[2] = {nullptr, nullptr};  // population buffers, swapped every step
    int cur = 0;
    void* F = nullptr;                // force field (double for F64 storage, float otherwise)
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
    int* vert_particle = nullptr;         // vertex -> particle
    int max_nv = 0;
    bool particles_dirty = true;  // host copies below are authoritative until uploaded
    std::vector<double> host_pos;    // concatenated vertex positions
    std::vector<double> host_stats;  // STATS per particle
    size_t membrane_smem = 0;
    int handle = -1;
};

// ---- kernel launchers (lattice_kernels.cu) ----
void launch_collide_stream(const Lattice& L, cudaStream_t s);
void launch_fd_walls(const Lattice& L, void* f, cudaStream_t s);
void launch_velocity(const Lattice& L, double* u, cudaStream_t s);
void launch_init_equilibrium(const Lattice& L, void* f, const double* rho, const double* u, cudaStream_t s);
void launch_import_soa(const Lattice& L, void* f, const double* src, cudaStream_t s);
void launch_export_soa(const Lattice& L, const void* f, double* dst, cudaStream_t s);
void launch_force_import(const Lattice& L, const double* src, cudaStream_t s);
void launch_force_export(const Lattice& L, double* dst, cudaStream_t s);
void launch_phase_import(const Lattice& L, const double* src, cudaStream_t s);
void launch_force_fill(const Lattice& L, cudaStream_t s);
void launch_nan_scan(const Lattice& L, int* flag, cudaStream_t s);

// ---- kernel launchers (ib_kernels.cu) ----
void launch_interpolate(const Lattice& L, cudaStream_t s);
void launch_membrane(const Lattice& L, cudaStream_t s);
void launch_spread(const Lattice& L, cudaStream_t s);
size_t membrane_smem_bytes(int max_nv);
void configure_membrane_kernel(size_t smem);

}  // namespace bib
