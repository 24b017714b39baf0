// Shared-memory staged collide-and-stream (the default kernel where the row fits).
//
// The lattice is cut into tiles of R consecutive x-rows of one z-plane (R * nx cells).
// For every tile, the source row segment of each of the 19 populations is one contiguous
// run of memory: rows (y - c_y, z - c_z) for y in the tile, or, behind a halfway
// bounce-back wall, the tile's own rows of the opposite population, or the wall buffer on
// finite-difference wall rows.  One warp per CTA moves these runs, and the tile's force
// rows, into shared memory with bulk asynchronous copies (cp.async.bulk) that complete on
// an mbarrier; the CTA is persistent and double-buffered, so the copies of tile t+1 are in
// flight while tile t is collided.  The whole memory-level parallelism sits in the copy
// engine instead of in registers, and every thread is left with shared-memory reads
// (the +-1 x shift is an index offset, periodic in x), FP32 arithmetic and coalesced stores.
//
// Per lattice update the kernel moves exactly the algorithmic bytes: 19 populations read
// and written once, the spread force read, and (coupled step) the previous force read,
// reset to the body force and the velocity field written.
#include <algorithm>
#include <mutex>
#include <unordered_map>

#include "lattice_common.cuh"

namespace bib {

namespace {

constexpr int kStagedThreads = 256;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for one phase of a stage barrier: gives up after about 2 s (a copy of a
// tile takes microseconds), so that a lost completion can never hang the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 26); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 0 && global_ns() - t0 > 2000000000ull) break;
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

// Collision of one cell in storage units.  FP32 compute with BGK(+Guo) uses the compact
// pairwise form; TRT and FP64 unscale, run the generic operator and rescale.  With u
// non-null the velocity j/rho + Fp/2 of the incoming state is returned.
template <class C, int COLL>
__device__ __forceinline__ void staged_collide(C* f, const C* F, C om, C omm, C S, C invS, const C* Fp, C* u) {
    if constexpr (sizeof(C) == 4 && COLL != BIB_COLLISION_TRT) {
        collide_compact<COLL>(f, F, om, S, invS, Fp, u);
    } else {
        if (sizeof(C) == 4) {
#pragma unroll
            for (int i = 0; i < Q; ++i) f[i] *= invS;
        }
        if (u) velocity_with_force(f, Fp, u);
        collide<C, COLL>(f, F, om, omm);
        if (sizeof(C) == 4) {
#pragma unroll
            for (int i = 0; i < Q; ++i) f[i] *= S;
        }
    }
}

struct StagedGeom {
    int R;            // rows per tile (divides ny)
    int Ct;           // cells per tile, R * nx
    int tiles_y;      // ny / R
    int64_t ntiles;   // tiles_y * nz
    unsigned pop_bytes, f_bytes;     // one population / force component of one tile
    unsigned off_fcol, off_fprev;    // byte offsets inside a stage
    unsigned stage_bytes, tx_bytes;  // stage size (padded) and bytes copied per tile
};

// Issue the copies of one tile into one stage (executed by warp 0).
template <class T, class FT, bool COUPLED, bool NEED_FCOL>
__device__ __forceinline__ void issue_tile(const LatticeDesc& d, const StagedGeom& g, int64_t tile, unsigned char* stage,
                                           uint64_t* bar, const T* fin, const T* wall, const FT* Fcol, const FT* Fprev,
                                           int lane) {
    const int z = (int)(tile / g.tiles_y);
    const int y0 = (int)(tile - (int64_t)z * g.tiles_y) * g.R;
    if (lane == 0) mbar_arrive_expect_tx(bar, g.tx_bytes);
    __syncwarp();
    const unsigned rowb = (unsigned)d.nx * sizeof(T);
    if (lane < Q) {
        const int i = lane;
        unsigned char* dst = stage + (size_t)i * g.pop_bytes;
        const unsigned char* run = nullptr;
        unsigned run_len = 0, run_at = 0;
        for (int r = 0; r < g.R; ++r) {
            const int y = y0 + r;
            const T* src;
            if (fd_wall_node(d, y)) {
                src = wall + i * wall_stride(d) + wall_index(d, y == 0 ? 0 : 1, 0, z);
            } else {
                int64_t srow;
                const int face = source_row(d, i, y, z, srow);
                src = face >= 0 ? fin + opposite(i) * d.stride + ((int64_t)y + (int64_t)d.ny * z) * d.nx
                                : fin + i * d.stride + srow * d.nx;
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
    } else {
        const int64_t row0 = ((int64_t)y0 + (int64_t)d.ny * z) * d.nx;
        if (NEED_FCOL && lane < Q + 3) {
            const int c = lane - Q;
            bulk_copy_g2s(stage + g.off_fcol + c * g.f_bytes, Fcol + c * d.stride + row0, g.f_bytes, bar);
        } else if (COUPLED && lane >= Q + 3 && lane < Q + 6) {
            const int c = lane - Q - 3;
            bulk_copy_g2s(stage + g.off_fprev + c * g.f_bytes, Fprev + c * d.stride + row0, g.f_bytes, bar);
        }
    }
}

template <class T, bool COUPLED, int COLL>
__global__ void __launch_bounds__(kStagedThreads, sizeof(T) == 8 ? 1 : 3) k_collide_stream_staged(
    LatticeDesc d, StagedGeom g, const T* __restrict__ fin, T* __restrict__ fout, const T* __restrict__ wall,
    const typename Store<T>::F* __restrict__ Fcol, typename Store<T>::F* __restrict__ Fprev,
    typename Store<T>::F* __restrict__ u_out, const uint8_t* __restrict__ phase, int* __restrict__ wait_err) {
    using C = typename Store<T>::C;
    using FT = typename Store<T>::F;
    constexpr bool NEED_FCOL = COLL == BIB_COLLISION_BGK_GUO_VOF;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_ok;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    unsigned char* stages = smem + 128;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int64_t tile = blockIdx.x;
    if (tile >= g.ntiles) return;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (warp == 0)
        issue_tile<T, FT, COUPLED, NEED_FCOL>(d, g, tile, stages, &bar[0], fin, wall, Fcol, Fprev, lane);

    const C S = sizeof(T) == 2 ? (C)d.scale : C(1);
    const C invS = sizeof(T) == 2 ? (C)d.inv_scale : C(1);
    C omm = C(0);
    if (COLL == BIB_COLLISION_TRT) {
        const C om = (C)d.omega;
        omm = C(1) / ((C)d.trt_magic / (C(1) / om - C(0.5)) + C(0.5));
    }
    for (int it = 0; tile < g.ntiles; ++it, tile += gridDim.x) {
        const int s = it & 1;
        const int64_t next = tile + gridDim.x;
        if (warp == 0 && next < g.ntiles)
            issue_tile<T, FT, COUPLED, NEED_FCOL>(d, g, next, stages + (s ^ 1) * g.stage_bytes, &bar[s ^ 1], fin, wall,
                                                  Fcol, Fprev, lane);
        if (tid == 0) {
            const bool ok = mbar_wait_bounded(&bar[s], (unsigned)(it >> 1) & 1u);
            if (!ok) {
                atomicExch(wait_err, 1);
                // let the copies of the prefetched tile land before the CTA leaves
                if (next < g.ntiles) mbar_wait_bounded(&bar[s ^ 1], (unsigned)((it + 1) >> 1) & 1u);
            }
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) return;  // uniform: every thread of the CTA leaves

        const unsigned char* st = stages + s * g.stage_bytes;
        const T* P = reinterpret_cast<const T*>(st);
        const FT* SFc = reinterpret_cast<const FT*>(st + g.off_fcol);
        const FT* SFp = reinterpret_cast<const FT*>(st + g.off_fprev);
        const int z = (int)(tile / g.tiles_y);
        const int y0 = (int)(tile - (int64_t)z * g.tiles_y) * g.R;
        for (int c = tid; c < g.Ct; c += kStagedThreads) {
            const int r = c / d.nx;
            const int x = c - r * d.nx;
            const int y = y0 + r;
            const int rb = r * d.nx;
            const int xl = x == 0 ? d.nx - 1 : x - 1;
            const int xr = x == d.nx - 1 ? 0 : x + 1;
            C f[Q];
            const bool fd = fd_wall_node(d, y);
            if (!row_special(d, y, z)) {
#pragma unroll
                for (int i = 0; i < Q; ++i)
                    f[i] = Staged<T>::one(P + i * g.Ct + rb + (cx(i) == 0 ? x : (cx(i) == 1 ? xl : xr)));
            } else {
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    int face = -1;
                    if (!fd) {
                        int64_t srow;
                        face = source_row(d, i, y, z, srow);
                    }
                    const bool shift = !fd && face < 0;
                    f[i] = Staged<T>::one(P + i * g.Ct + rb + (!shift || cx(i) == 0 ? x : (cx(i) == 1 ? xl : xr)));
                    if (face >= 0) f[i] += moving_wall_term<C>(d, i, face) * S;
                }
            }
            const int64_t k = ((int64_t)y + (int64_t)d.ny * z) * d.nx + x;
            C F[3] = {C(0), C(0), C(0)};
            if (NEED_FCOL) {
#pragma unroll
                for (int q = 0; q < 3; ++q) F[q] = (C)SFc[q * g.Ct + c];
            }
            C om = (C)d.omega;
            if (COLL == BIB_COLLISION_BGK_GUO_VOF) {
                om = (C)d.omega_c0;
                if (d.use_phase && phase[k]) om = (C)d.omega_c1;
            }
            if (COUPLED) {
                C Fp[3], u[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) Fp[q] = (C)SFp[q * g.Ct + c];
                staged_collide<C, COLL>(f, F, om, omm, S, invS, Fp, fd ? nullptr : u);
                if (fd) {
                    const int side = y == 0 ? 0 : 1;
#pragma unroll
                    for (int q = 0; q < 3; ++q) u[q] = (C)d.wall_u[side][q];
                }
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    u_out[q * d.stride + k] = (FT)u[q];
                    Fprev[q * d.stride + k] = (FT)d.body[q];
                }
            } else {
                staged_collide<C, COLL>(f, F, om, omm, S, invS, nullptr, nullptr);
            }
#pragma unroll
            for (int i = 0; i < Q; ++i) Staged<T>::put(fout + i * d.stride + k, f[i]);
        }
        __syncthreads();  // the stage is refilled in the next-but-one iteration
    }
}

// Rows per tile: the largest divisor R of ny with R * nx <= target cells.
int staged_rows(const LatticeDesc& d, int target) {
    int R = 1;
    for (int r = 1; r <= d.ny; ++r)
        if (d.ny % r == 0 && (int64_t)r * d.nx <= target) R = r;
    return R;
}


template <class T>
size_t staged_geom(const LatticeDesc& d, int target, bool coupled, bool need_fcol, StagedGeom& g) {
    using FT = typename Store<T>::F;
    g = StagedGeom{};
    g.R = staged_rows(d, target);
    g.Ct = g.R * d.nx;
    g.tiles_y = d.ny / g.R;
    g.ntiles = (int64_t)g.tiles_y * d.nz;
    g.pop_bytes = (unsigned)(g.Ct * sizeof(T));
    g.f_bytes = (unsigned)(g.Ct * sizeof(FT));
    g.off_fcol = Q * g.pop_bytes;
    g.off_fprev = g.off_fcol + (need_fcol ? 3 * g.f_bytes : 0);
    g.tx_bytes = g.off_fprev + (coupled ? 3 * g.f_bytes : 0);
    g.stage_bytes = (g.tx_bytes + 127) / 128 * 128;
    return 128 + 2 * (size_t)g.stage_bytes;
}

bool smem_fits(size_t smem) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return smem + 1024 <= (size_t)optin;
}

int default_tile_cells(const Lattice& L) {
    return L.tile_cells > 0 ? L.tile_cells : (L.storage == BIB_STORAGE_F64 ? 256 : 512);
}

template <class T, bool COUPLED, int COLL>
bool staged_inst(const Lattice& L, int target, cudaStream_t s) {
    using FT = typename Store<T>::F;
    constexpr bool NEED_FCOL = COLL == BIB_COLLISION_BGK_GUO_VOF;
    const LatticeDesc& d = L.d;
    StagedGeom g;
    const size_t smem = staged_geom<T>(d, target, COUPLED, NEED_FCOL, g);
    if (!smem_fits(smem)) return false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);

    auto kern = k_collide_stream_staged<T, COUPLED, COLL>;
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
        if (r == 0 && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, kStagedThreads, smem) != cudaSuccess ||
                       r < 1)) {
            r = 0;
            return false;
        }
        nb = r;
    }
    const int64_t grid = std::min<int64_t>(g.ntiles, (int64_t)nb * sms);
    const T* fin = (const T*)L.f[L.cur];
    T* fout = (T*)L.f[1 - L.cur];
    const FT* Fcol = (const FT*)(COUPLED ? L.F[1 - L.fe] : L.F[L.fe]);
    FT* Fprev = COUPLED ? (FT*)L.F[L.fe] : nullptr;
    kern<<<(unsigned)grid, kStagedThreads, smem, s>>>(d, g, fin, fout, (const T*)L.wall, Fcol, Fprev,
                                                       COUPLED ? (FT*)L.u : nullptr, L.phase, L.wait_err);
    return true;
}

template <class T, bool COUPLED>
bool staged_coll(const Lattice& L, int target, cudaStream_t s) {
    switch (L.d.collision) {
        case BIB_COLLISION_BGK_GUO_VOF: return staged_inst<T, COUPLED, BIB_COLLISION_BGK_GUO_VOF>(L, target, s);
        case BIB_COLLISION_BGK: return staged_inst<T, COUPLED, BIB_COLLISION_BGK>(L, target, s);
        default: return staged_inst<T, COUPLED, BIB_COLLISION_TRT>(L, target, s);
    }
}

template <class T>
bool shape_ok(const Lattice& L) {
    return L.d.nx % 2 == 0 && (L.d.nx * sizeof(T)) % 16 == 0;
}

template <class T>
bool staged_t(const Lattice& L, bool coupled, cudaStream_t s) {
    if (!shape_ok<T>(L) || !L.wait_err) return false;
    const int target = default_tile_cells(L);
    return coupled ? staged_coll<T, true>(L, target, s) : staged_coll<T, false>(L, target, s);
}

template <class T>
bool fits_t(const Lattice& L) {
    if (!shape_ok<T>(L)) return false;
    StagedGeom g;
    return smem_fits(staged_geom<T>(L.d, default_tile_cells(L), true, true, g));  // the largest stage
}

}  // namespace

bool collide_staged_fits(const Lattice& L) {
    if (L.storage == BIB_STORAGE_F64) return fits_t<double>(L);
    if (L.storage == BIB_STORAGE_F32) return fits_t<float>(L);
    return fits_t<__half>(L);
}

bool launch_collide_stream_staged(const Lattice& L, bool coupled, cudaStream_t s) {
    if (L.storage == BIB_STORAGE_F64) return staged_t<double>(L, coupled, s);
    if (L.storage == BIB_STORAGE_F32) return staged_t<float>(L, coupled, s);
    return staged_t<__half>(L, coupled, s);
}

}  // namespace bib
