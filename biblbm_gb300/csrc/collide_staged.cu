// Shared-memory staged collide-and-stream (the default kernel where the row fits).
//
// The lattice is cut into tiles of R consecutive x-rows of one z-plane (R * nx cells).
// For every tile, the source row segment of each of the 19 populations is one contiguous
// run of memory: rows (y - c_y, z - c_z) for y in the tile, or, behind a halfway
// bounce-back wall, the tile's own rows of the opposite population, or the wall buffer on
// finite-difference wall rows.  One warp per CTA moves these runs, and the tile's force
// rows, into shared memory with bulk asynchronous copies (cp.async.bulk) that complete on
// an mbarrier; the CTA is persistent with a ring of 2..8 stages (3 for FP16, two CTAs per SM;
// 4 for FP32 / FP64), so the copies of the next tiles are in flight while a tile is collided.
// The memory-level parallelism sits in the bulk-copy engine instead of in registers, and every
// thread is left with shared-memory reads (the +-1 x shift is an index offset, periodic in x),
// arithmetic in FP32 (FP64 for FP64 storage) and coalesced stores.
//
// Per lattice update the kernel moves exactly the algorithmic bytes: 19 populations read
// and written once, the spread force read, the velocity field written (coupled step) and, with
// the dense coupling only, the previous force read and reset to the body force.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "lattice_common.cuh"

namespace bib {

namespace {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// One potentially blocking test of a barrier phase: a thread whose phase is not complete is
// suspended until it completes or about kSuspendNs pass (the suspend-time hint), so that waiting
// warps do not spin through issue slots the working warps need.
constexpr uint32_t kSuspendNs = 20000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for one phase of a stage barrier: gives up after limit_ns (2 s by default; a
// copy of a tile takes microseconds) or 2^26 polls, so that a lost completion can never hang
// the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, uint64_t limit_ns = kDefaultWaitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 26); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 0 && global_ns() - t0 > limit_ns) break;
    }
    return false;
}
// Global -> shared bulk copy; dst, src and bytes are multiples of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Values of a staged population row as the compute type, in storage units (FP16 keeps the
// scaled f-bar; the scale is folded into the collision).
template <class T>
struct Staged;
template <>
struct Staged<__half> {
    static __device__ __forceinline__ float one(const __half* p) { return __half2float(*p); }
    static __device__ __forceinline__ void two(const __half* p, float& a, float& b) {
        const float2 v = __half22float2(*reinterpret_cast<const __half2*>(p));
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void store(__half* p, float a, float b) {
        *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
    }
    static __device__ __forceinline__ void put(__half* p, float a) { *p = __float2half_rn(a); }
};
template <>
struct Staged<float> {
    static __device__ __forceinline__ float one(const float* p) { return *p; }
    static __device__ __forceinline__ void two(const float* p, float& a, float& b) {
        const float2 v = *reinterpret_cast<const float2*>(p);
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void store(float* p, float a, float b) {
        *reinterpret_cast<float2*>(p) = make_float2(a, b);
    }
    static __device__ __forceinline__ void put(float* p, float a) { *p = a; }
};
template <>
struct Staged<double> {
    static __device__ __forceinline__ double one(const double* p) { return *p; }
    static __device__ __forceinline__ void two(const double* p, double& a, double& b) {
        const double2 v = *reinterpret_cast<const double2*>(p);
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void store(double* p, double a, double b) {
        *reinterpret_cast<double2*>(p) = make_double2(a, b);
    }
    static __device__ __forceinline__ void put(double* p, double a) { *p = a; }
};

// The 19 post-collision values of one cell to their arrays (stride apart); FP16 converts two
// values per instruction (same rounding; measured on the 400-cell channel: the collide-and-stream
// 0.1763 -> 0.1748 ms, the lattice-only TRT kernel 56,680 -> 57,370 MLUPS at 384^3).
template <class T, class C>
__device__ __forceinline__ void store_cell(T* o, int64_t stride, const C* f) {
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        Staged<T>::put(o, f[i]);
        o += stride;
    }
}
template <>
__device__ __forceinline__ void store_cell<__half, float>(__half* o, int64_t stride, const float* f) {
#pragma unroll
    for (int i = 0; i + 1 < Q; i += 2) {
        const __half2 h = __floats2half2_rn(f[i], f[i + 1]);
        o[0] = __low2half(h);
        o[stride] = __high2half(h);
        o += 2 * stride;
    }
    *o = __float2half_rn(f[Q - 1]);
}

// Collision of one cell in storage units: the compact pairwise forms (BGK + Guo, BGK, TRT) in the
// compute type.  With u non-null the velocity j/rho + Fp/2 of the incoming state is returned.
template <class C, int COLL>
__device__ __forceinline__ void staged_relax(C* f, const C* F, C om, C omm, C S, const CellMoments<C>& m) {
    if constexpr (COLL == BIB_COLLISION_TRT) {
        const C Fm[3] = {omm, C(0), C(0)};  // the TRT branch takes omega_minus in F[0]
        relax_compact<C, COLL>(f, Fm, om, S, m);
    } else {
        relax_compact<C, COLL>(f, F, om, S, m);
    }
}

// Tile pitch in cells: the shared-memory row of one population holds up to TILE cells, so
// every staged address is a per-thread base plus a compile-time offset.
template <class T>
struct TileOf {
    static constexpr int value = sizeof(T) == 8 ? 256 : 512;
};

// Coupling of a staged launch: lattice only; dense (the velocity field with the previous force,
// which is read and reset to the body force); sparse (the velocity field with the body force,
// the previous force left to the sparse reset).
constexpr int kCplNone = 0, kCplDense = 1, kCplSparse = 2;

// Stage layout (compile-time): 19 population rows, the collision force (BGK + Guo) and,
// for the dense coupled step, the previous force, each TILE cells long.
template <class T, int CPL, int COLL>
struct StageLayout {
    using FT = typename Store<T>::F;
    static constexpr int TILE = TileOf<T>::value;
    static constexpr int CONSUMERS = TILE / 32;  // consumer warps: one cell per thread and tile
    static constexpr int THREADS = 32 * (CONSUMERS + 1);
    static constexpr bool NEED_FCOL = COLL == BIB_COLLISION_BGK_GUO_VOF;
    static constexpr unsigned POP = TILE * sizeof(T);
    static constexpr unsigned FRC = TILE * sizeof(FT);
    static constexpr unsigned OFF_FCOL = Q * POP;
    static constexpr unsigned OFF_FPREV = OFF_FCOL + (NEED_FCOL ? 3 * FRC : 0);
    static constexpr unsigned BYTES = ((OFF_FPREV + (CPL == kCplDense ? 3 * FRC : 0)) + 127) / 128 * 128;
};

constexpr int kMaxStages = 8;

struct StagedGeom {
    int R;            // rows per tile (divides ny)
    int Ct;           // cells per tile, R * nx <= TILE
    int tiles_y;      // ny / R
    int nstages;      // pipeline depth (2..kMaxStages)
    int64_t ntiles;   // tiles_y * nz
    unsigned tx_bytes;  // bytes copied in per tile
    uint64_t wait_ns;   // bound of the hand-off waits (full / empty); the final drain keeps the default
    int64_t withhold;   // failure testing: a tile whose copies the producer does not issue (-1: none)
};

struct TileRef {
    int z, y0;
    int64_t row0;  // first cell of the tile
};
__device__ __forceinline__ TileRef tile_ref(const LatticeDesc& d, const StagedGeom& g, int64_t tile) {
    // tile indices of one lattice fit 32 bits (checked on the host): a 32-bit division is a
    // fraction of the 64-bit sequence, and every consumer thread evaluates it per tile
    const unsigned ti = (unsigned)tile, ty = (unsigned)g.tiles_y;
    TileRef t;
    t.z = (int)(ti / ty);
    t.y0 = (int)(ti - (unsigned)t.z * ty) * g.R;
    t.row0 = ((int64_t)t.y0 + (int64_t)d.ny * t.z) * d.nx;
    return t;
}

// Lattice vector of the population a producer lane moves, resolved once per kernel (the
// lane index is not a compile-time constant, so cx(i) etc. would be evaluated per row).
struct PopLane {
    int cy, cz, opp;
};
__device__ __forceinline__ PopLane pop_lane(int lane) {
    PopLane p{0, 0, 0};
#pragma unroll
    for (int i = 0; i < Q; ++i)
        if (lane == i) {
            p.cy = cy(i);
            p.cz = cz(i);
            p.opp = opposite(i);
        }
    return p;
}

// Copies of one tile into one stage, by the producer warp: lane i < 19 moves population i,
// lanes 19..21 the collision force, lanes 22..24 the previous force (dense coupling).
template <class T, int CPL, int COLL>
__device__ __forceinline__ void load_tile(const LatticeDesc& d, const StagedGeom& g, int64_t tile, unsigned char* stage,
                                          uint64_t* bar, const T* fin, const T* wall, const typename Store<T>::F* Fcol,
                                          const typename Store<T>::F* Fprev, int lane, const PopLane& pl) {
    using L = StageLayout<T, CPL, COLL>;
    using FT = typename Store<T>::F;
    const TileRef t = tile_ref(d, g, tile);
    if (lane == 0) mbar_arrive_expect_tx(bar, g.tx_bytes);
    __syncwarp();
    const unsigned rowb = (unsigned)d.nx * sizeof(T);
    if (lane < Q) {
        const int i = lane;
        unsigned char* dst = stage + i * L::POP;
        // source plane of this population (periodic wrap or a z wall behind it)
        int zs = t.z - pl.cz;
        bool zface = false;
        if (d.pz) zs = zs < 0 ? zs + d.nz : (zs >= d.nz ? zs - d.nz : zs);
        else zface = zs < 0 || zs >= d.nz;
        const int ya = t.y0 - pl.cy, yb = t.y0 + g.R - 1 - pl.cy;  // source rows of the tile's first / last row
        const bool fd_rows = d.fd_walls && (t.y0 == 0 || t.y0 + g.R == d.ny);
        if (!zface && !fd_rows && ya >= 0 && yb < d.ny) {
            // every row of the tile streams from the neighbouring rows of one plane: one run
            bulk_copy_g2s(dst, fin + i * d.stride + ((int64_t)ya + (int64_t)d.ny * zs) * d.nx, g.R * rowb, bar);
        } else {
            const unsigned char* run = nullptr;
            unsigned run_len = 0, run_at = 0;
            for (int r = 0; r < g.R; ++r) {
                const int y = t.y0 + r;
                const T* src;
                if (fd_wall_node(d, y)) {
                    src = wall + i * wall_stride(d) + wall_index(d, y == 0 ? 0 : 1, 0, t.z);
                } else {
                    int ys = y - pl.cy;
                    bool face = zface;
                    if (d.py) ys = ys < 0 ? ys + d.ny : (ys >= d.ny ? ys - d.ny : ys);
                    else face = face || ys < 0 || ys >= d.ny;
                    src = face ? fin + pl.opp * d.stride + ((int64_t)y + (int64_t)d.ny * t.z) * d.nx
                               : fin + i * d.stride + ((int64_t)ys + (int64_t)d.ny * zs) * d.nx;
                }
                const unsigned char* s = reinterpret_cast<const unsigned char*>(src);
                if (run_len && s == run + run_len) {
                    run_len += rowb;
                } else {
                    if (run_len) bulk_copy_g2s(dst + run_at, run, run_len, bar);
                    run = s;
                    run_len = rowb;
                    run_at = (unsigned)r * rowb;
                }
            }
            bulk_copy_g2s(dst + run_at, run, run_len, bar);
        }
    } else {
        const unsigned fb = (unsigned)(g.Ct * sizeof(FT));
        if (L::NEED_FCOL && lane < Q + 3) {
            const int c = lane - Q;
            bulk_copy_g2s(stage + L::OFF_FCOL + c * L::FRC, Fcol + c * d.stride + t.row0, fb, bar);
        } else if (CPL == kCplDense && lane >= Q + 3 && lane < Q + 6) {
            const int c = lane - Q - 3;
            bulk_copy_g2s(stage + L::OFF_FPREV + c * L::FRC, Fprev + c * d.stride + t.row0, fb, bar);
        }
    }
    __syncwarp();
}

// Consumer side of one tile: the thread's cell of every tile and its x-neighbours (periodic in
// x within the row).
struct TileCell {
    bool active;
    int r, o0, ol, orr;
};
__device__ __forceinline__ TileCell tile_cell(const LatticeDesc& d, int Ct, int ct) {
    TileCell c;
    c.active = ct < Ct;
    c.r = ct / d.nx;
    const int x = ct - c.r * d.nx;
    c.o0 = ct;
    c.ol = c.r * d.nx + (x == 0 ? d.nx - 1 : x - 1);
    c.orr = c.r * d.nx + (x == d.nx - 1 ? 0 : x + 1);
    return c;
}

// Collision and stores of one cell k of row y whose gathered populations are in f: a
// BounceBack / NoDynamics node is not collided (zero velocity), every other node collides with
// the force F; the coupled step writes its velocity (j/rho + Fp/2, or the wall's on
// finite-difference wall rows) and, with the dense coupling, resets the previous force.
template <class T, int CPL, int COLL>
__device__ __forceinline__ void finish_cell(const LatticeDesc& d, const CollideParams<typename Store<T>::C>& cp,
                                            T* __restrict__ fout, typename Store<T>::F* __restrict__ Fprev,
                                            typename Store<T>::U* __restrict__ u_out, const uint8_t* __restrict__ phase,
                                            const uint8_t* __restrict__ celltype, int64_t k, int y, bool fd,
                                            typename Store<T>::C* f, const typename Store<T>::C* F,
                                            const typename Store<T>::C* Fp) {
    using C = typename Store<T>::C;
    using FT = typename Store<T>::F;
    using UT = typename Store<T>::U;
    const int ctype = d.has_types ? celltype[k] : BIB_CELL_FLUID;
    if (ctype != BIB_CELL_FLUID) {  // BounceBack / NoDynamics node: no collision, zero velocity
        if (CPL != kCplNone) store_u<UT>(u_out, k, (UT)0.0f, (UT)0.0f, (UT)0.0f);
        if (CPL == kCplDense) {
#pragma unroll
            for (int q = 0; q < 3; ++q) Fprev[q * d.stride + k] = (FT)cp.body[q];
        }
        if (ctype == BIB_CELL_BOUNCE_BACK) bounce_back_cell(f);
        store_cell<T, C>(fout + k, d.stride, f);
        return;
    }
    C om = cp.om0;
    if (COLL == BIB_COLLISION_BGK_GUO_VOF && d.use_phase && phase[k]) om = cp.om1;
    const CellMoments<C> m = moments_compact<C>(f, cp.invS);
    if (CPL != kCplNone) {
        // the velocity and the force reset are stored before the relaxation, so that the
        // previous force is dead while the relaxation runs
        C u[3];
        if (fd) {
            const int side = y == 0 ? 0 : 1;
#pragma unroll
            for (int q = 0; q < 3; ++q) u[q] = cp.wall_u[side][q];
        } else {
            velocity_compact<C>(m, Fp, u);
        }
        store_u_from<UT, C>(u_out, k, u[0], u[1], u[2]);
        if (CPL == kCplDense) {
#pragma unroll
            for (int q = 0; q < 3; ++q) Fprev[q * d.stride + k] = (FT)cp.body[q];
        }
    }
    staged_relax<C, COLL>(f, F, om, cp.omm, cp.S, m);
    store_cell<T, C>(fout + k, d.stride, f);
}

// One cell per consumer thread: read the thread's cell from the stage, release the stage,
// collide and store.
template <class T, int CPL, int COLL>
__device__ __forceinline__ void consume_cell(const LatticeDesc& d, const StagedGeom& g, int64_t tile, const unsigned char* st,
                                             const CollideParams<typename Store<T>::C>& cp, T* __restrict__ fout,
                                             typename Store<T>::F* __restrict__ Fprev, typename Store<T>::U* __restrict__ u_out,
                                             const uint8_t* __restrict__ phase, const uint8_t* __restrict__ celltype,
                                             const TileCell& cell, uint64_t* empty_s, int lane) {
    using C = typename Store<T>::C;
    using FT = typename Store<T>::F;
    using L = StageLayout<T, CPL, COLL>;
    constexpr int TILE = L::TILE;
    const int r = cell.r, o0 = cell.o0, ol = cell.ol, orr = cell.orr;
    const bool active = cell.active;
    const T* P = reinterpret_cast<const T*>(st);
    const FT* SFc = reinterpret_cast<const FT*>(st + L::OFF_FCOL);
    const FT* SFp = reinterpret_cast<const FT*>(st + L::OFF_FPREV);
    const TileRef t = tile_ref(d, g, tile);
    C f[Q], F[3] = {C(0), C(0), C(0)}, Fp[3] = {C(0), C(0), C(0)};
    const int y = t.y0 + r;
    const bool fd = fd_wall_node(d, y);
    if (active) {
        if (!row_special(d, y, t.z)) {
#pragma unroll
            for (int i = 0; i < Q; ++i) f[i] = Staged<T>::one(P + i * TILE + (cx(i) == 0 ? o0 : (cx(i) == 1 ? ol : orr)));
        } else {
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                int face = -1;
                if (!fd) {
                    int64_t srow;
                    face = source_row(d, i, y, t.z, srow);
                }
                const bool shift = !fd && face < 0;
                f[i] = Staged<T>::one(P + i * TILE + (!shift || cx(i) == 0 ? o0 : (cx(i) == 1 ? ol : orr)));
                if (face >= 0) f[i] += cp.mw[face][i];
            }
        }
        if (L::NEED_FCOL) {
#pragma unroll
            for (int q = 0; q < 3; ++q) F[q] = (C)SFc[q * TILE + o0];
        }
        if (CPL == kCplDense) {
#pragma unroll
            for (int q = 0; q < 3; ++q) Fp[q] = (C)SFp[q * TILE + o0];
        } else if (CPL == kCplSparse) {
#pragma unroll
            for (int q = 0; q < 3; ++q) Fp[q] = cp.body[q];
        }
    }
    // the stage has been read into registers: hand it back to the producer
    __syncwarp();
    if (lane == 0) mbar_arrive(empty_s);
    if (!active) return;
    finish_cell<T, CPL, COLL>(d, cp, fout, Fprev, u_out, phase, celltype, t.row0 + o0, y, fd, f, F, Fp);
}

// The consumer of one tile.
template <class T, int CPL, int COLL>
__device__ __forceinline__ void consume_tile(const LatticeDesc& d, const StagedGeom& g, int64_t tile, const unsigned char* st,
                                             const CollideParams<typename Store<T>::C>& cp, T* __restrict__ fout,
                                             typename Store<T>::F* __restrict__ Fprev, typename Store<T>::U* __restrict__ u_out,
                                             const uint8_t* __restrict__ phase, const uint8_t* __restrict__ celltype,
                                             const TileCell& cell, uint64_t* empty_s, int lane) {
    consume_cell<T, CPL, COLL>(d, g, tile, st, cp, fout, Fprev, u_out, phase, celltype, cell, empty_s, lane);
}

// Warp-specialised persistent kernel: warp 0 produces, warps 1..CONSUMERS collide.  Stage
// s is handed over through two mbarriers: full[s] completes when the tile's bytes have
// landed, empty[s] when every consumer warp is done reading it.  Consumers never wait for
// each other, and the producer refills a stage as soon as it is released, so up to NS - 1
// tiles of loads are in flight per CTA.  Results go straight from registers to HBM.
// Resident CTAs per SM the kernel is built for: FP16 needs two (32 consumer warps) to hide
// the latency of its arithmetic; FP32 and FP64 run one CTA with a deeper pipeline.
template <class T>
constexpr int staged_ctas_per_sm() {
    return sizeof(T) == 2 ? 2 : 1;
}

template <class T, int CPL, int COLL>
__global__ void __launch_bounds__(StageLayout<T, CPL, COLL>::THREADS, staged_ctas_per_sm<T>())
    k_collide_stream_staged(
    LatticeDesc d, StagedGeom g, CollideParams<typename Store<T>::C> cp, const T* __restrict__ fin,
    T* __restrict__ fout, const T* __restrict__ wall, const typename Store<T>::F* __restrict__ Fcol,
    typename Store<T>::F* __restrict__ Fprev, typename Store<T>::U* __restrict__ u_out,
    const uint8_t* __restrict__ phase, const uint8_t* __restrict__ celltype, int* __restrict__ wait_err) {
    using C = typename Store<T>::C;
    using FT = typename Store<T>::F;
    using L = StageLayout<T, CPL, COLL>;
    constexpr int TILE = L::TILE;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);
    uint64_t* empty = full + kMaxStages;
    unsigned char* stages = smem + 256;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int NS = g.nstages;
    if ((int64_t)blockIdx.x >= g.ntiles) return;
    if (tid == 0) {
        for (int k = 0; k < NS; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], L::CONSUMERS);
        }
        mbar_init_fence();
    }
    __syncthreads();

    if (warp == 0) {
        // ---- producer
        const PopLane pl = pop_lane(lane);
        int it = 0, withheld = -1;
        for (int64_t tile = blockIdx.x; tile < g.ntiles; tile += gridDim.x, ++it) {
            const int s = it % NS, use = it / NS;
            if (use > 0) {
                // every lane observes the release, so every lane's copies are ordered after it
                const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&empty[s], (unsigned)(use - 1) & 1u, g.wait_ns));
                if (!ok) {
                    if (lane == 0) atomicExch(wait_err, 1);
                    break;
                }
            }
            if (tile == g.withhold) {  // failure testing: this stage's phase is never completed
                withheld = it;
                continue;
            }
            load_tile<T, CPL, COLL>(d, g, tile, stages + s * L::BYTES, &full[s], fin, wall, Fcol, Fprev, lane, pl);
        }
        // a copy may still be landing only if the consumers gave up; wait for it so that
        // no bulk copy writes into the shared memory of a retired CTA (a withheld tile has none)
        if (lane == 0) {
            const int issued = it;
            for (int k = issued > NS ? issued - NS : 0; k < issued; ++k)
                if (k != withheld) mbar_wait_bounded(&full[k % NS], (unsigned)(k / NS) & 1u);
        }
        return;
    }

    // ---- consumers: thread `ct` owns cell ct of every tile
    const TileCell cell = tile_cell(d, g.Ct, tid - 32);
    int it = 0;
    for (int64_t tile = blockIdx.x; tile < g.ntiles; tile += gridDim.x, ++it) {
        const int s = it % NS;
        // every lane waits, so that the landed bytes are visible to every lane
        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[s], (unsigned)(it / NS) & 1u, g.wait_ns));
        if (!ok) {
            if (lane == 0) atomicExch(wait_err, 1);
            return;
        }
        consume_tile<T, CPL, COLL>(d, g, tile, stages + s * L::BYTES, cp, fout, Fprev, u_out, phase, celltype, cell,
                                        &empty[s], lane);
    }
}

// Batched variant: the global tile index runs over the tiles of all lattices of a batch
// (CollideView::tile0 is the first tile of each); producer and consumers look the lattice
// of each tile up in the view table (coupled step only).
__device__ __forceinline__ int find_view(const CollideView* __restrict__ views, int n, int64_t tile) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (views[mid].tile0 <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ StagedGeom view_geom(const CollideView& v, int ns) {
    StagedGeom g;
    g.R = v.R;
    g.Ct = v.Ct;
    g.tiles_y = v.tiles_y;
    g.nstages = ns;
    g.ntiles = v.ntiles;
    g.tx_bytes = v.tx_bytes;
    g.wait_ns = kDefaultWaitNs;
    g.withhold = -1;
    return g;
}

// Shared memory of the batched kernel after its stages: the producer's and the consumers'
// copies of the current lattice view (the view table outgrows L1 next to the stages, and its
// fields would otherwise be L2 round trips on every tile) and the first tile of every view.
constexpr int kMaxCachedViews = 512;
__host__ __device__ constexpr size_t batch_extra_smem() {
    return 2 * sizeof(CollideView) + kMaxCachedViews * sizeof(int64_t);
}

// View of `tile`: tiles of a CTA only grow, so step forward from the previous one
__device__ __forceinline__ int next_view(const int64_t* tile0, int n, int vi, int64_t tile) {
    while (vi + 1 < n && tile0[vi + 1] <= tile) ++vi;
    return vi;
}

// Copy a view into shared memory with `nthreads` threads starting at thread `t`.
__device__ __forceinline__ void copy_view(CollideView* dst, const CollideView* src, int t, int nthreads) {
    static_assert(sizeof(CollideView) % 16 == 0, "views copy as 16-byte words");
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (int k = t; k < (int)(sizeof(CollideView) / 16); k += nthreads) d4[k] = s4[k];
}

template <class T, int COLL>
__global__ void __launch_bounds__(StageLayout<T, kCplDense, COLL>::THREADS, staged_ctas_per_sm<T>())
    k_collide_stream_staged_batch(const CollideView* __restrict__ views, int nviews, int64_t ntiles, int NS,
                                  int* __restrict__ wait_err) {
    using C = typename Store<T>::C;
    using FT = typename Store<T>::F;
    using L = StageLayout<T, kCplDense, COLL>;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);
    uint64_t* empty = full + kMaxStages;
    unsigned char* stages = smem + 256;
    CollideView* pview = reinterpret_cast<CollideView*>(stages + (size_t)NS * L::BYTES);
    CollideView* cview = pview + 1;
    int64_t* tile0 = reinterpret_cast<int64_t*>(cview + 1);
    const bool cached = nviews <= kMaxCachedViews;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if ((int64_t)blockIdx.x >= ntiles) return;
    if (tid == 0) {
        for (int k = 0; k < NS; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], L::CONSUMERS);
        }
        mbar_init_fence();
    }
    if (cached)
        for (int k = tid; k < nviews; k += blockDim.x) tile0[k] = views[k].tile0;
    __syncthreads();
    if (warp == 0) {
        const PopLane pl = pop_lane(lane);
        int it = 0, vi = 0, have = -1;
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
            const int s = it % NS, use = it / NS;
            if (use > 0) {
                const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&empty[s], (unsigned)(use - 1) & 1u));
                if (!ok) {
                    if (lane == 0) atomicExch(wait_err, 1);
                    break;
                }
            }
            vi = cached ? next_view(tile0, nviews, vi, tile) : find_view(views, nviews, tile);
            if (vi != have) {
                copy_view(pview, views + vi, lane, 32);
                __syncwarp();
                have = vi;
            }
            const CollideView& V = *pview;
            load_tile<T, kCplDense, COLL>(V.d, view_geom(V, NS), tile - V.tile0, stages + s * L::BYTES, &full[s],
                                     static_cast<const T*>(V.fin), static_cast<const T*>(V.wall),
                                     static_cast<const FT*>(V.Fcol), static_cast<const FT*>(V.Fprev), lane, pl);
        }
        if (lane == 0) {
            const int issued = it;
            for (int k = issued > NS ? issued - NS : 0; k < issued; ++k)
                mbar_wait_bounded(&full[k % NS], (unsigned)(k / NS) & 1u);
        }
        return;
    }
    int it = 0, cur_view = -1, vi = 0;
    TileCell cell{};
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int s = it % NS;
        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[s], (unsigned)(it / NS) & 1u));
        if (!ok) {
            if (lane == 0) atomicExch(wait_err, 1);
            return;
        }
        vi = cached ? next_view(tile0, nviews, vi, tile) : find_view(views, nviews, tile);
        if (vi != cur_view) {
            // every consumer is done with the previous view before it is replaced (named
            // barrier 1 spans the consumer warps only; they all visit the same tiles)
            asm volatile("bar.sync 1, %0;" ::"r"(L::CONSUMERS * 32) : "memory");
            copy_view(cview, views + vi, tid - 32, L::CONSUMERS * 32);
            asm volatile("bar.sync 1, %0;" ::"r"(L::CONSUMERS * 32) : "memory");
            cell = tile_cell(cview->d, cview->Ct, tid - 32);  // depends on the lattice's row length
            cur_view = vi;
        }
        const CollideView& V = *cview;
        consume_tile<T, kCplDense, COLL>(V.d, view_geom(V, NS), tile - V.tile0, stages + s * L::BYTES,
                                    *reinterpret_cast<const CollideParams<C>*>(V.cp), static_cast<T*>(V.fout),
                                    static_cast<FT*>(V.Fprev), static_cast<typename Store<T>::U*>(V.u), V.phase, V.celltype, cell,
                                    &empty[s], lane);
    }
}

// Rows per tile: the largest divisor R of ny with R * nx <= target cells.
int staged_rows(const LatticeDesc& d, int target) {
    int R = 1;
    for (int r = 1; r <= d.ny; ++r)
        if (d.ny % r == 0 && (int64_t)r * d.nx <= target) R = r;
    return R;
}

int optin_smem() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return optin;
}

template <class T, int CPL, int COLL>
size_t staged_smem(int nstages) {
    return 256 + (size_t)nstages * StageLayout<T, CPL, COLL>::BYTES;
}

// Pipeline depth: the tuning value, else as many stages as fit the resident CTAs of an SM
// (228 KB of shared memory per SM, 1 KB of it reserved per CTA).
template <class T, int CPL, int COLL>
int staged_stages(const Lattice& L) {
    if (L.stages >= 2) return L.stages;
    const size_t limit = std::min<size_t>((size_t)optin_smem(), 228 * 1024 / staged_ctas_per_sm<T>()) - 1024;
    int best = 2;
    for (int ns = 2; ns <= kMaxStages; ++ns)
        if (staged_smem<T, CPL, COLL>(ns) <= limit) best = ns;
    return best;
}

template <class C>
CollideParams<C> collide_params(const LatticeDesc& d, int storage) {
    CollideParams<C> cp{};
    const bool phase_omega = d.collision == BIB_COLLISION_BGK_GUO_VOF;
    cp.om0 = (C)(phase_omega ? d.omega_c0 : d.omega);
    cp.om1 = (C)(phase_omega ? d.omega_c1 : d.omega);
    cp.omm = (C)(1.0 / (d.trt_magic / (1.0 / d.omega - 0.5) + 0.5));
    const double S = storage == BIB_STORAGE_F16 ? (double)d.scale : 1.0;
    cp.S = (C)S;
    cp.invS = (C)(storage == BIB_STORAGE_F16 ? (double)d.inv_scale : 1.0);
    for (int q = 0; q < 3; ++q) {
        cp.body[q] = (C)d.body[q];
        cp.wall_u[0][q] = (C)d.wall_u[0][q];
        cp.wall_u[1][q] = (C)d.wall_u[1][q];
    }
    for (int face = 0; face < 4; ++face)
        for (int i = 0; i < Q; ++i) {
            const double cu = cx(i) * d.wall_u[face][0] + cy(i) * d.wall_u[face][1] + cz(i) * d.wall_u[face][2];
            cp.mw[face][i] = (C)((C)(6.0 * weight<double>(i) * cu) * (C)S);
        }
    return cp;
}

template <class T, int CPL, int COLL>
bool staged_inst(const Lattice& L, int target, cudaStream_t s) {
    using FT = typename Store<T>::F;
    using C = typename Store<T>::C;
    using LY = StageLayout<T, CPL, COLL>;
    const LatticeDesc& d = L.d;
    StagedGeom g{};
    g.R = staged_rows(d, std::min(target, LY::TILE));
    g.Ct = g.R * d.nx;
    if (g.Ct > LY::TILE) return false;
    g.tiles_y = d.ny / g.R;
    g.ntiles = (int64_t)g.tiles_y * d.nz;
    g.nstages = staged_stages<T, CPL, COLL>(L);
    g.wait_ns = L.wait_ns;
    g.withhold = L.withhold_tile;
    g.tx_bytes = (unsigned)(Q * g.Ct * sizeof(T) + ((LY::NEED_FCOL ? 3 : 0) + (CPL == kCplDense ? 3 : 0)) * g.Ct * sizeof(FT));
    const size_t smem = staged_smem<T, CPL, COLL>(g.nstages);
    if (smem + 1024 > (size_t)optin_smem()) return false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);

    auto kern = k_collide_stream_staged<T, CPL, COLL>;
    // per device: the dynamic shared memory this kernel is allowed (only ever raised) and
    // the resident CTAs per SM for each stage size
    static std::mutex mu;
    static std::unordered_map<int, size_t> allowed;
    static std::unordered_map<int64_t, int> resident;
    int nb = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        size_t& lim = allowed[dev];
        if (smem > lim) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return false;
            lim = smem;
        }
        int& r = resident[((int64_t)dev << 32) | (int64_t)smem];
        if (r == 0 && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, LY::THREADS, smem) != cudaSuccess ||
                       r < 1)) {
            r = 0;
            return false;
        }
        nb = r;
    }
    const int64_t grid = std::min<int64_t>(g.ntiles, (int64_t)nb * sms);
    const T* fin = (const T*)L.f[L.cur];
    T* fout = (T*)L.f[1 - L.cur];
    const FT* Fcol = (const FT*)(CPL != kCplNone ? L.F[1 - L.fe] : L.F[L.fe]);
    FT* Fprev = CPL == kCplDense ? (FT*)L.F[L.fe] : nullptr;
    kern<<<(unsigned)grid, LY::THREADS, smem, s>>>(d, g, collide_params<C>(d, L.storage), fin, fout,
                                                       (const T*)L.wall, Fcol, Fprev, CPL != kCplNone ? (typename Store<T>::U*)L.u : nullptr,
                                                       L.phase, L.celltype, L.wait_err);
    return true;
}

template <class T, int CPL>
bool staged_coll(const Lattice& L, int target, cudaStream_t s) {
    switch (L.d.collision) {
        case BIB_COLLISION_BGK_GUO_VOF: return staged_inst<T, CPL, BIB_COLLISION_BGK_GUO_VOF>(L, target, s);
        case BIB_COLLISION_BGK: return staged_inst<T, CPL, BIB_COLLISION_BGK>(L, target, s);
        default: return staged_inst<T, CPL, BIB_COLLISION_TRT>(L, target, s);
    }
}

template <class T>
bool shape_ok(const Lattice& L) {
    // tiles are whole x-rows; their count per lattice (at most ny * nz) must fit 31 bits
    return L.d.nx % 2 == 0 && (L.d.nx * sizeof(T)) % 16 == 0 && L.d.nx <= TileOf<T>::value &&
           (int64_t)L.d.ny * L.d.nz < ((int64_t)1 << 31);
}

int default_tile_cells(const Lattice& L) {
    return L.tile_cells > 0 ? L.tile_cells : (L.storage == BIB_STORAGE_F64 ? 256 : 512);
}

template <class T>
bool staged_t(const Lattice& L, Coupling mode, cudaStream_t s) {
    if (!shape_ok<T>(L) || !L.wait_err) return false;
    const int target = default_tile_cells(L);
    switch (mode) {
        case Coupling::kDense: return staged_coll<T, kCplDense>(L, target, s);
        case Coupling::kSparse: return staged_coll<T, kCplSparse>(L, target, s);
        default: return staged_coll<T, kCplNone>(L, target, s);
    }
}

template <class T>
bool fits_t(const Lattice& L) {
    if (!shape_ok<T>(L)) return false;
    const int ns = L.stages >= 2 ? L.stages : 2;
    return ns <= kMaxStages && staged_smem<T, kCplDense, BIB_COLLISION_BGK_GUO_VOF>(ns) + 1024 <= (size_t)optin_smem();
}

template <class T, int COLL>
bool batch_inst(const BatchLaunch& B, cudaStream_t s) {
    using LY = StageLayout<T, kCplDense, COLL>;
    const int ns = B.stages >= 2 ? B.stages : staged_stages<T, kCplDense, COLL>(Lattice{});
    const size_t smem = staged_smem<T, kCplDense, COLL>(ns) + batch_extra_smem();
    if (smem + 1024 > (size_t)optin_smem()) return false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto kern = k_collide_stream_staged_batch<T, COLL>;
    static std::mutex mu;
    static std::unordered_map<int, size_t> allowed;
    static std::unordered_map<int64_t, int> resident;
    int nb = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        size_t& lim = allowed[dev];
        if (smem > lim) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return false;
            lim = smem;
        }
        int& r = resident[((int64_t)dev << 32) | (int64_t)smem];
        if (r == 0 && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, LY::THREADS, smem) != cudaSuccess ||
                       r < 1)) {
            r = 0;
            return false;
        }
        nb = r;
    }
    const int64_t grid = std::min<int64_t>(B.ntiles, (int64_t)nb * sms);
    kern<<<(unsigned)grid, LY::THREADS, smem, s>>>(B.cviews, B.n, B.ntiles, ns, B.wait_err);
    return true;
}

template <class T>
bool batch_t(const BatchLaunch& B, cudaStream_t s) {
    switch (B.collision) {
        case BIB_COLLISION_BGK_GUO_VOF: return batch_inst<T, BIB_COLLISION_BGK_GUO_VOF>(B, s);
        case BIB_COLLISION_BGK: return batch_inst<T, BIB_COLLISION_BGK>(B, s);
        default: return batch_inst<T, BIB_COLLISION_TRT>(B, s);
    }
}

template <class T>
bool view_t(const Lattice& L, int tile_cells, CollideView& v) {
    using FT = typename Store<T>::F;
    using C = typename Store<T>::C;
    if (!shape_ok<T>(L)) return false;
    const LatticeDesc& d = L.d;
    const int target = std::min(tile_cells > 0 ? tile_cells : (sizeof(T) == 8 ? 256 : 512), TileOf<T>::value);
    v.d = d;
    v.R = staged_rows(d, target);
    v.Ct = v.R * d.nx;
    if (v.Ct > TileOf<T>::value) return false;
    v.tiles_y = d.ny / v.R;
    v.ntiles = (int64_t)v.tiles_y * d.nz;
    const bool need_fcol = d.collision == BIB_COLLISION_BGK_GUO_VOF;
    v.tx_bytes = (unsigned)(Q * v.Ct * sizeof(T) + ((need_fcol ? 3 : 0) + 3) * v.Ct * sizeof(FT));
    const CollideParams<C> cp = collide_params<C>(d, L.storage);
    static_assert(sizeof(CollideParams<C>) <= sizeof(v.cp), "collision constants fit the view");
    std::memcpy(v.cp, &cp, sizeof(cp));
    return true;
}

}  // namespace

bool staged_collide_view(const Lattice& L, int tile_cells, CollideView& v) {
    if (L.storage == BIB_STORAGE_F64) return view_t<double>(L, tile_cells, v);
    if (L.storage == BIB_STORAGE_F32) return view_t<float>(L, tile_cells, v);
    return view_t<__half>(L, tile_cells, v);
}

bool collide_batch_fits(int storage, int collision, int stages) {
    auto fits = [&](auto tag) {
        using T = decltype(tag);
        const int ns = stages >= 2 ? stages : 2;
        size_t smem = 0;
        if (collision == BIB_COLLISION_BGK_GUO_VOF) smem = staged_smem<T, kCplDense, BIB_COLLISION_BGK_GUO_VOF>(ns);
        else if (collision == BIB_COLLISION_BGK) smem = staged_smem<T, kCplDense, BIB_COLLISION_BGK>(ns);
        else smem = staged_smem<T, kCplDense, BIB_COLLISION_TRT>(ns);
        return ns <= 4 && smem + batch_extra_smem() + 1024 <= (size_t)optin_smem();
    };
    if (storage == BIB_STORAGE_F64) return fits(double{});
    if (storage == BIB_STORAGE_F32) return fits(float{});
    return fits(__half{});
}

bool launch_collide_batch(const BatchLaunch& B, cudaStream_t s) {
    if (B.n == 0 || B.ntiles == 0) return true;
    if (B.storage == BIB_STORAGE_F64) return batch_t<double>(B, s);
    if (B.storage == BIB_STORAGE_F32) return batch_t<float>(B, s);
    return batch_t<__half>(B, s);
}

bool collide_staged_fits(const Lattice& L) {
    if (L.storage == BIB_STORAGE_F64) return fits_t<double>(L);
    if (L.storage == BIB_STORAGE_F32) return fits_t<float>(L);
    return fits_t<__half>(L);
}

bool launch_collide_stream_staged(const Lattice& L, Coupling mode, cudaStream_t s) {
    if (L.storage == BIB_STORAGE_F64) return staged_t<double>(L, mode, s);
    if (L.storage == BIB_STORAGE_F32) return staged_t<float>(L, mode, s);
    return staged_t<__half>(L, mode, s);
}

}  // namespace bib
