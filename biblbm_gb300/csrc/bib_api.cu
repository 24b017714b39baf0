// Host runtime behind the C ABI (include/bib/bib.h): contexts, lattices, shapes,
// particles, the coupled step and its CUDA-graph replay.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "bib_internal.h"

using namespace bib;

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int cur = 0, pcur = 0;
    int kernels = 0;  // kernel nodes of the captured graph
};

struct Batch;

struct bib_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<std::unique_ptr<Lattice>> lattices;
    std::vector<std::unique_ptr<ShapeHost>> shapes;
    bool graph_mode = true;
    bool profiling = false;
    double prof[5] = {0, 0, 0, 0, 0};  // membrane, spread, collide+stream, walls, interpolate+update
    cudaEvent_t ev[6] = {};
    cudaEvent_t dl_ev[8] = {};  // completion of the asynchronous downloads, one per slot
    int* d_flag = nullptr;
    void* spread_scratch = nullptr;  // device address of the no-allocation spreading's static array
    std::map<std::pair<int, int>, GraphEntry> graphs;  // (lattice, steps and parity) -> step graph
    // population transfers with pageable host buffers: two device staging halves filled and
    // drained on a copy stream while the import / export kernels work on the other half
    double* stage = nullptr;
    size_t stage_count = 0;   // size of both halves in doubles
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t tx_ready[2] = {}, tx_free[2] = {}, tx_start = nullptr;
    // device allocations made so far, and the index of one that is made to fail (the
    // environment variable BIB_FAIL_DEVICE_ALLOC at bib_create; -1: none), for failure tests
    int64_t alloc_count = 0, fail_alloc = -1;
    std::vector<std::unique_ptr<Batch>> batches;
    ~bib_ctx();
};

namespace {

bib_status fail(bib_ctx* c, bib_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return s;
}

#define BIB_CUDA(ctx, expr)                                                                               \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess) return fail(ctx, BIB_ECUDA, "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                           \
    } while (0)

#define BIB_CHECK_LAUNCH(ctx) BIB_CUDA(ctx, cudaGetLastError())

// Every device allocation of a context: cudaMalloc, except the one that BIB_FAIL_DEVICE_ALLOC
// names, which fails as an exhausted device would (cudaErrorMemoryAllocation).
cudaError_t dev_malloc(bib_ctx* c, void** p, size_t bytes) {
    const int64_t k = c->alloc_count++;
    if (k == c->fail_alloc) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

#define BIB_ALLOC(ctx, ptr, bytes)                                                                        \
    do {                                                                                                  \
        const size_t b_ = (bytes);                                                                        \
        cudaError_t e_ = dev_malloc(ctx, (void**)(ptr), b_);                                              \
        if (e_ != cudaSuccess) {                                                                          \
            cudaGetLastError();                                                                           \
            return fail(ctx, BIB_ENOMEM, "device allocation of %zu bytes failed (%s:%d): %s", b_, __FILE__, \
                        __LINE__, cudaGetErrorString(e_));                                                \
        }                                                                                                 \
    } while (0)

Lattice* get_lattice(bib_ctx* c, int32_t h) {
    if (!c || h < 0 || h >= (int32_t)c->lattices.size() || !c->lattices[h]) return nullptr;
    return c->lattices[h].get();
}

size_t pop_bytes(int storage) { return storage == BIB_STORAGE_F64 ? 8 : (storage == BIB_STORAGE_F32 ? 4 : 2); }
size_t force_bytes(int storage) { return storage == BIB_STORAGE_F64 ? 8 : 4; }
// one value of the velocity field (FP16 for FP16 populations)
size_t velocity_bytes(int storage) { return storage == BIB_STORAGE_F64 ? 8 : (storage == BIB_STORAGE_F32 ? 4 : 2); }

// ---------------------------------------------------------------- shapes
// ParticleShape constructor and compute_connectivity, src/fsi/ParticleShape.hh:21-212:
// triangle rest areas (tri::normal_and_area), total area, signed volume, unique links in
// (min, max) vertex order with their rest length, and for every link shared by two
// triangles the adjacent pair (i0, i1, i2, i3) with (i0,i1,i2) and (i0,i2,i3) the two
// triangles and the cosine / sine of the rest dihedral angle.
struct V3d {
    double x, y, z;
};
inline V3d sub(V3d a, V3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3d crs(V3d a, V3d b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dt(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double nrm(V3d a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3d scl(V3d a, double s) { return {a.x / s, a.y / s, a.z / s}; }

bool build_shape(ShapeHost& S, const double* xyz, const int64_t* tri, int64_t nv, int64_t nt, std::string& why) {
    S.rest.assign(xyz, xyz + 3 * nv);
    S.tri.resize(3 * nt);
    for (int64_t i = 0; i < 3 * nt; ++i) {
        if (tri[i] < 0 || tri[i] >= nv) {
            why = "triangle index out of range";
            return false;
        }
        S.tri[i] = (int)tri[i];
    }
    auto P = [&](int i) { return V3d{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}; };
    S.tri_area.resize(nt);
    S.area = 0;
    S.volume = 0;
    for (int64_t t = 0; t < nt; ++t) {
        V3d a = P(S.tri[3 * t]), b = P(S.tri[3 * t + 1]), c = P(S.tri[3 * t + 2]);
        double ar = nrm(crs(sub(b, a), sub(c, a))) * 0.5;
        if (!(ar > 0)) {
            why = "degenerate triangle";
            return false;
        }
        S.tri_area[t] = ar;
        S.area += ar;
        S.volume += dt(a, crs(b, c)) / 6.;
    }
    struct L {
        int t1 = -1, t2 = -1;
        double len = 0;
    };
    std::map<std::pair<int, int>, L> links;
    for (int64_t t = 0; t < nt; ++t) {
        int ind[4] = {S.tri[3 * t], S.tri[3 * t + 1], S.tri[3 * t + 2], S.tri[3 * t]};
        for (int j = 0; j < 3; ++j) {
            std::pair<int, int> key(std::min(ind[j], ind[j + 1]), std::max(ind[j], ind[j + 1]));
            auto it = links.find(key);
            if (it == links.end()) {
                L l;
                l.t1 = (int)t;
                l.len = nrm(sub(P(key.first), P(key.second)));
                links.emplace(key, l);
            } else if (it->second.t1 != (int)t) {
                it->second.t2 = (int)t;
            }
        }
    }
    S.links.clear();
    S.link_len.clear();
    S.pairs.clear();
    S.pair_cs.clear();
    for (auto& kv : links) {
        const int i0 = kv.first.first, i1 = kv.first.second;
        S.links.push_back(i0);
        S.links.push_back(i1);
        S.link_len.push_back(kv.second.len);
        if (kv.second.t1 < 0 || kv.second.t2 < 0) continue;
        int a[3] = {S.tri[3 * kv.second.t1], S.tri[3 * kv.second.t1 + 1], S.tri[3 * kv.second.t1 + 2]};
        int b[3] = {S.tri[3 * kv.second.t2], S.tri[3 * kv.second.t2 + 1], S.tri[3 * kv.second.t2 + 2]};
        for (int g = 0; g < 3 && !((a[0] == i0 && a[2] == i1) || (a[0] == i1 && a[2] == i0)); ++g) {
            int tmp = a[0]; a[0] = a[2]; a[2] = a[1]; a[1] = tmp;
        }
        for (int g = 0; g < 3 && !((b[0] == i0 && b[1] == i1) || (b[0] == i1 && b[1] == i0)); ++g) {
            int tmp = b[0]; b[0] = b[2]; b[2] = b[1]; b[1] = tmp;
        }
        const int q[4] = {a[0], a[1], a[2], b[2]};
        for (int k = 0; k < 4; ++k) S.pairs.push_back(q[k]);
        V3d p0 = P(q[0]), p1 = P(q[1]), p2 = P(q[2]), p3 = P(q[3]);
        V3d n1 = crs(sub(p1, p0), sub(p2, p0));
        n1 = scl(n1, nrm(n1));
        V3d n2 = crs(sub(p2, p0), sub(p3, p0));
        n2 = scl(n2, nrm(n2));
        S.pair_cs.push_back(dt(n1, n2));
        S.pair_cs.push_back((dt(sub(n1, n2), sub(p1, p3)) > 0 ? 1.0 : -1.0) * nrm(crs(n1, n2)));
    }
    // FP32 copies of the rest-state constants for the reduced-precision element kernels
    S.tri_rest_f.resize(4 * nt);
    S.tri_area_f.resize(nt);
    for (int64_t t = 0; t < nt; ++t) {
        const V3d a = P(S.tri[3 * t]), b = P(S.tri[3 * t + 1]), c = P(S.tri[3 * t + 2]);
        const V3d e0 = sub(b, a), e1 = sub(c, a);
        const double l0 = nrm(e0), l0p = nrm(e1);
        S.tri_rest_f[4 * t] = (float)l0;
        S.tri_rest_f[4 * t + 1] = (float)l0p;
        S.tri_rest_f[4 * t + 2] = (float)(dt(e0, e1) / (l0 * l0p));
        S.tri_rest_f[4 * t + 3] = (float)(nrm(crs(e0, e1)) / (l0 * l0p));
        S.tri_area_f[t] = (float)S.tri_area[t];
    }
    S.pair_cs_f.assign(S.pair_cs.begin(), S.pair_cs.end());
    S.tri4.assign(4 * nt, 0);
    for (int64_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k) S.tri4[4 * t + k] = S.tri[3 * t + k];
    // per-vertex incidence lists for the deterministic force gather: links, then triangles,
    // then pairs, each in element order (the order of the reference's element loops)
    std::vector<std::vector<int>> incv(nv);
    const int nl = (int)S.link_len.size(), np = (int)S.pair_cs.size() / 2;
    for (int l = 0; l < nl; ++l)
        for (int k = 0; k < 2; ++k) incv[S.links[2 * l + k]].push_back((0 << 29) | l);
    for (int t = 0; t < (int)nt; ++t)
        for (int k = 0; k < 3; ++k) incv[S.tri[3 * t + k]].push_back((1 << 29) | t);
    for (int q = 0; q < np; ++q)
        for (int k = 0; k < 4; ++k) incv[S.pairs[4 * q + k]].push_back((2 << 29) | q);
    S.inc_off.assign(1, 0);
    S.inc.clear();
    for (int64_t v = 0; v < nv; ++v) {
        S.inc.insert(S.inc.end(), incv[v].begin(), incv[v].end());
        S.inc_off.push_back((int)S.inc.size());
    }
    // a spatially clustered visiting order of the vertices (Morton order of the rest shape on a
    // unit grid): neighbouring threads of the interpolation then gather from neighbouring rows
    // (measured 0.0558 -> 0.0534 ms on the 400-cell channel; the spreading does not gain)
    double lo[3] = {xyz[0], xyz[1], xyz[2]};
    for (int64_t v = 0; v < nv; ++v)
        for (int a = 0; a < 3; ++a) lo[a] = std::min(lo[a], xyz[3 * v + a]);
    std::vector<std::pair<uint64_t, int>> code((size_t)nv);
    for (int64_t v = 0; v < nv; ++v) {
        uint64_t m = 0;
        for (int a = 0; a < 3; ++a) {
            const uint64_t q = (uint64_t)std::min(std::max(std::floor(xyz[3 * v + a] - lo[a]), 0.0), 1048575.0);
            for (int b = 0; b < 20; ++b) m |= ((q >> b) & 1u) << (3 * b + a);
        }
        code[(size_t)v] = {m, (int)v};
    }
    std::stable_sort(code.begin(), code.end(), [](const std::pair<uint64_t, int>& a, const std::pair<uint64_t, int>& b) {
        return a.first < b.first;
    });
    S.order.resize((size_t)nv);
    for (int64_t v = 0; v < nv; ++v) S.order[(size_t)v] = code[(size_t)v].second;
    return true;
}

template <class T>
bib_status upload(bib_ctx* c, T** dptr, const std::vector<T>& v) {
    *dptr = nullptr;
    if (v.empty()) return BIB_OK;
    BIB_ALLOC(c, (void**)dptr, v.size() * sizeof(T));
    BIB_CUDA(c, cudaMemcpy(*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return BIB_OK;
}

// DeformableParticle3D::update (DeformableParticle3D.hh:54-82) on the host, FP64.
void particle_update(const ShapeHost& S, const double* pos, double* st) {
    double area = 0, vol = 0, cx = 0, cy = 0, cz = 0;
    const int nt = (int)S.tri_area.size();
    for (int t = 0; t < nt; ++t) {
        const double* a = pos + 3 * S.tri[3 * t];
        const double* b = pos + 3 * S.tri[3 * t + 1];
        const double* c = pos + 3 * S.tri[3 * t + 2];
        V3d A{a[0], a[1], a[2]}, B{b[0], b[1], b[2]}, C{c[0], c[1], c[2]};
        const double dA = nrm(crs(sub(B, A), sub(C, A))) * 0.5;
        area += dA;
        vol += dt(A, crs(B, C)) / 6.;
        cx += (A.x + B.x + C.x) / 3.0 * dA;
        cy += (A.y + B.y + C.y) / 3.0 * dA;
        cz += (A.z + B.z + C.z) / 3.0 * dA;
    }
    st[0] = area;
    st[1] = vol;
    st[2] = cx / area;
    st[3] = cy / area;
    st[4] = cz / area;
}

// ParticleBase3D::map_center_of_mass_to_periodic_grid (ParticleBase.hh:111-136)
void remap_com(const LatticeDesc& d, double* pos, int nv, double* st) {
    const int N[3] = {d.nx, d.ny, d.nz};
    const int per[3] = {d.px, d.py, d.pz};
    double delta[3] = {0, 0, 0};
    for (int a = 0; a < 3; ++a) {
        if (!per[a]) continue;
        const double L = (double)N[a], Linv = 1. / L;
        const double np_ = st[2 + a] - L * std::floor((st[2 + a] - (-0.5)) * Linv);
        delta[a] = np_ - st[2 + a];
        st[2 + a] = np_;
    }
    if (delta[0] != 0 || delta[1] != 0 || delta[2] != 0)
        for (int i = 0; i < nv; ++i)
            for (int a = 0; a < 3; ++a) pos[3 * i + a] += delta[a];
}

// DeformableParticle3D::compute_moment_of_intertia, DeformableParticle3D.hh:173-272
void moment_of_inertia(const ShapeHost& S, const double* pos, double* I) {
    double in[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int nt = (int)S.tri_area.size();
    for (int t = 0; t < nt; ++t) {
        const double* v0 = pos + 3 * S.tri[3 * t];
        const double* v1 = pos + 3 * S.tri[3 * t + 1];
        const double* v2 = pos + 3 * S.tri[3 * t + 2];
        V3d N = crs(V3d{v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]}, V3d{v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]});
        double f1[3], f2[3], f3[3], g0[3], g1[3], g2[3];
        for (int d = 0; d < 3; ++d) {
            double tmp0 = v0[d] + v1[d];
            f1[d] = tmp0 + v2[d];
            double tmp1 = v0[d] * v0[d];
            double tmp2 = tmp1 + v1[d] * tmp0;
            f2[d] = tmp2 + v2[d] * f1[d];
            f3[d] = v0[d] * tmp1 + v1[d] * tmp2 + v2[d] * f2[d];
            g0[d] = f2[d] + v0[d] * (f1[d] + v0[d]);
            g1[d] = f2[d] + v1[d] * (f1[d] + v1[d]);
            g2[d] = f2[d] + v2[d] * (f1[d] + v2[d]);
        }
        in[0] += N.x * f1[0];
        in[1] += N.x * f2[0];
        in[2] += N.y * f2[1];
        in[3] += N.z * f2[2];
        in[4] += N.x * f3[0];
        in[5] += N.y * f3[1];
        in[6] += N.z * f3[2];
        in[7] += N.x * (v0[1] * g0[0] + v1[1] * g1[0] + v2[1] * g2[0]);
        in[8] += N.y * (v0[2] * g0[1] + v1[2] * g1[1] + v2[2] * g2[1]);
        in[9] += N.z * (v0[0] * g0[2] + v1[0] * g1[2] + v2[0] * g2[2]);
    }
    in[0] *= 1.0 / 6.0;
    for (int k = 1; k <= 3; ++k) in[k] *= 1.0 / 24.0;
    for (int k = 4; k <= 6; ++k) in[k] *= 1.0 / 60.0;
    for (int k = 7; k <= 9; ++k) in[k] *= 1.0 / 120.0;
    const double vol = in[0];
    const double c[3] = {in[1] / vol, in[2] / vol, in[3] / vol};
    I[0] = in[5] + in[6] - vol * (c[1] * c[1] + c[2] * c[2]);
    I[1] = -in[7] + vol * c[0] * c[1];
    I[2] = -in[9] + vol * c[2] * c[0];
    I[3] = I[1];
    I[4] = in[4] + in[6] - vol * (c[2] * c[2] + c[0] * c[0]);
    I[5] = -in[8] + vol * c[1] * c[2];
    I[6] = I[2];
    I[7] = I[5];
    I[8] = in[4] + in[5] - vol * (c[0] * c[0] + c[1] * c[1]);
}

// The force fields were written outside the sparse coupled step: neither may be reset by its
// recorded support nodes any more (the next reset of each is a dense fill).
void forces_touched(Lattice& L) { L.sparse_ok[0] = L.sparse_ok[1] = false; }

// The coupled step resets the previous force field sparsely (only where the spreading wrote)
// when the tuning asks for it, on reduced-precision lattices whose velocity field near the
// membranes is j/rho + F/2 at every node: no phase field, cell types, second-order walls or pipe
// boundary.
bool sparse_coupling(const Lattice& L) {
    return L.sparse_reset && L.storage != BIB_STORAGE_F64 && L.nvert > 0 && !L.phase && !L.celltype && L.nguo == 0 &&
           !L.ib.has_pipe && L.spread_lo[0] && L.spread_lo[1];
}

void free_particles(Lattice& L) {
    for (int k = 0; k < 2; ++k) {
        cudaFree(L.pos[k]);
        L.pos[k] = nullptr;
    }
    cudaFree(L.vel);
    cudaFree(L.force);
    cudaFree(L.stats);
    cudaFree(L.upd_partial);
    L.upd_partial = nullptr;
    for (int k = 0; k < 2; ++k) {
        cudaFree(L.spread_lo[k]);
        L.spread_lo[k] = nullptr;
    }
    forces_touched(L);
    cudaFree(L.pdev);
    cudaFree(L.vert_particle);
    cudaFree(L.visit_order);
    L.visit_order = nullptr;
    L.vel = L.force = L.stats = nullptr;
    L.pdev = nullptr;
    L.vert_particle = nullptr;
    for (int k = 0; k < 2; ++k) {
        cudaFree(L.sort_keys[k]);
        cudaFree(L.sort_ids[k]);
        L.sort_keys[k] = L.sort_ids[k] = nullptr;
    }
    cudaFree(L.sort_temp);
    L.sort_temp = nullptr;
    L.sort_temp_bytes = 0;
    for (int k = 0; k < 2; ++k) {
        cudaFree(L.pgrid.keys[k]);
        cudaFree(L.pgrid.ids[k]);
    }
    cudaFree(L.pgrid.start);
    cudaFree(L.pgrid.end);
    cudaFree(L.pgrid.temp);
    L.pgrid = PairGrid{};
    for (int k = 0; k < 2; ++k) {
        cudaFree(L.rgrid.keys[k]);
        cudaFree(L.rgrid.ids[k]);
    }
    cudaFree(L.rgrid.start);
    cudaFree(L.rgrid.end);
    cudaFree(L.rgrid.posf);
    cudaFree(L.rgrid.temp);
    L.rgrid = RefGridBuffers{};
    cudaFree(L.vox_count);
    cudaFree(L.vox_z);
    L.vox_count = nullptr;
    L.vox_z = nullptr;
}

void drop_graphs(bib_ctx* c, int32_t h) {
    for (auto it = c->graphs.begin(); it != c->graphs.end();) {
        if (it->first.first == h) {
            if (it->second.exec) cudaGraphExecDestroy(it->second.exec);
            it = c->graphs.erase(it);
        } else {
            ++it;
        }
    }
}

bib_status sync_particles(bib_ctx* c, Lattice& L) {
    if (!L.particles_dirty) return BIB_OK;
    ++L.version;
    free_particles(L);
    L.nvert = (int)(L.host_pos.size() / 3);
    const int np = (int)L.parts.size();
    if (np == 0) {
        L.particles_dirty = false;
        return BIB_OK;
    }
    const size_t vb = 3 * (size_t)L.nvert * sizeof(double);
    for (int k = 0; k < 2; ++k) BIB_ALLOC(c, (void**)&L.pos[k], vb);
    BIB_ALLOC(c, (void**)&L.vel, vb);
    BIB_ALLOC(c, (void**)&L.force, vb);
    BIB_ALLOC(c, (void**)&L.stats, STATS * np * sizeof(double));
    BIB_ALLOC(c, (void**)&L.upd_partial, (size_t)np * 64 * 5 * sizeof(double));
    for (int k = 0; k < 2; ++k) BIB_ALLOC(c, (void**)&L.spread_lo[k], (size_t)L.nvert * sizeof(int4));
    forces_touched(L);
    BIB_CUDA(c, cudaMemcpy(L.pos[0], L.host_pos.data(), vb, cudaMemcpyHostToDevice));
    BIB_CUDA(c, cudaMemcpy(L.pos[1], L.host_pos.data(), vb, cudaMemcpyHostToDevice));
    BIB_CUDA(c, cudaMemset(L.vel, 0, vb));
    BIB_CUDA(c, cudaMemset(L.force, 0, vb));
    BIB_CUDA(c, cudaMemcpy(L.stats, L.host_stats.data(), STATS * np * sizeof(double), cudaMemcpyHostToDevice));
    L.pcur = 0;
    std::vector<ParticleDev> pd(np);
    L.max_nv = 0;
    L.max_elems = 0;
    L.max_nt = 0;
    for (int p = 0; p < np; ++p) {
        const ParticleHost& ph = L.parts[p];
        const ShapeHost& S = *c->shapes[ph.shape];
        ParticleDev& d = pd[p];
        d.shape = ph.shape;
        d.model = ph.model;
        d.v0 = ph.v0;
        d.nv = ph.nv;
        d.nt = (int)S.tri_area.size();
        d.nl = (int)S.link_len.size();
        d.np = (int)S.pair_cs.size() / 2;
        d.rest = S.dev.rest;
        d.tri = S.dev.tri;
        d.tri_area = S.dev.tri_area;
        d.links = S.dev.links;
        d.link_len = S.dev.link_len;
        d.pairs = S.dev.pairs;
        d.pair_cs = S.dev.pair_cs;
        d.inc_off = S.dev.inc_off;
        d.inc = S.dev.inc;
        d.tri_rest_f = S.dev.tri_rest_f;
        d.tri4 = S.dev.tri4;
        d.tri_area_f = S.dev.tri_area_f;
        d.pair_cs_f = S.dev.pair_cs_f;
        d.inst = 0;
        d.lpid = p;
        d.A0 = S.area;
        for (int k = 0; k < BIB_P_COUNT; ++k) d.prm[k] = ph.prm[k];
        L.max_nv = std::max(L.max_nv, ph.nv);
        L.max_elems = std::max(L.max_elems, std::max(d.nt, std::max(d.nl, d.np)));
        L.max_nt = std::max(L.max_nt, d.nt);
    }
    if (L.ib.spread_mode == BIB_SPREAD_DETERMINISTIC) {
        const int sup = L.ib.dirac == BIB_DIRAC_PESKIN ? 4 : 3;
        const int64_t ne = (int64_t)L.nvert * sup * sup * sup;
        if (ne >= (int64_t)1 << 31) return fail(c, BIB_EUNSUPPORTED, "too many spreading entries for the sort");
        for (int k = 0; k < 2; ++k) {
            BIB_ALLOC(c, (void**)&L.sort_keys[k], ne * sizeof(uint32_t));
            BIB_ALLOC(c, (void**)&L.sort_ids[k], ne * sizeof(uint32_t));
        }
        L.sort_temp_bytes = spread_sort_temp_bytes(ne);
        BIB_ALLOC(c, &L.sort_temp, L.sort_temp_bytes);
    }
    {
        std::vector<int> vp(L.nvert);
        for (int p = 0; p < np; ++p)
            for (int v = 0; v < L.parts[p].nv; ++v) vp[L.parts[p].v0 + v] = p;
        BIB_ALLOC(c, (void**)&L.vert_particle, L.nvert * sizeof(int));
        BIB_CUDA(c, cudaMemcpy(L.vert_particle, vp.data(), L.nvert * sizeof(int), cudaMemcpyHostToDevice));
        // the interpolation's visiting order: every particle's vertices in its shape's clustered order
        for (int p = 0; p < np; ++p) {
            const ShapeHost& S = *c->shapes[L.parts[p].shape];
            for (int v = 0; v < L.parts[p].nv; ++v) vp[L.parts[p].v0 + v] = L.parts[p].v0 + S.order[v];
        }
        BIB_ALLOC(c, (void**)&L.visit_order, L.nvert * sizeof(int));
        BIB_CUDA(c, cudaMemcpy(L.visit_order, vp.data(), L.nvert * sizeof(int), cudaMemcpyHostToDevice));
    }
    BIB_ALLOC(c, (void**)&L.pdev, np * sizeof(ParticleDev));
    BIB_CUDA(c, cudaMemcpy(L.pdev, pd.data(), np * sizeof(ParticleDev), cudaMemcpyHostToDevice));
    L.pdev_host = pd;
    L.membrane_smem = membrane_smem_bytes(L.max_nv);
    int dev_max = 0;
    BIB_CUDA(c, cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    if (L.membrane_smem + 1024 > (size_t)dev_max)
        return fail(c, BIB_EUNSUPPORTED, "mesh with %d vertices exceeds the membrane kernel's shared memory", L.max_nv);
    configure_membrane_kernel(L.membrane_smem);
    if (L.inter.npp > 0 && L.inter.pp_search == BIB_PAIR_SEARCH_GRID) {
        // the reference's collision grid over the lattice box: a dense table of its cells
        const int64_t box[6] = {0, L.d.nx - 1, 0, L.d.ny - 1, 0, L.d.nz - 1};
        const int per[3] = {L.d.px, L.d.py, L.d.pz};
        if (ref_grid_cells(box) > kMaxRefGridCells)
            return fail(c, BIB_EUNSUPPORTED, "lattice too large for the reference's collision grid");
        const RefGrid g = ref_grid(box, per, L.inter.pp_cut, L.nvert);
        RefGridBuffers& R = L.rgrid;
        R.bits = ref_grid_bits(g.ncell);
        for (int k = 0; k < 2; ++k) {
            BIB_ALLOC(c, (void**)&R.keys[k], L.nvert * sizeof(uint32_t));
            BIB_ALLOC(c, (void**)&R.ids[k], L.nvert * sizeof(uint32_t));
        }
        BIB_CUDA(c, cudaMemset(R.keys[1], 0, L.nvert * sizeof(uint32_t)));
        BIB_ALLOC(c, (void**)&R.posf, L.nvert * sizeof(float4));
        BIB_ALLOC(c, (void**)&R.start, ((size_t)g.ncell + 1) * sizeof(int));
        BIB_ALLOC(c, (void**)&R.end, ((size_t)g.ncell + 1) * sizeof(int));
        BIB_CUDA(c, cudaMemset(R.start, 0, ((size_t)g.ncell + 1) * sizeof(int)));
        BIB_CUDA(c, cudaMemset(R.end, 0, ((size_t)g.ncell + 1) * sizeof(int)));
        R.temp_bytes = ref_grid_temp_bytes(L.nvert, R.bits);
        BIB_ALLOC(c, &R.temp, std::max<size_t>(R.temp_bytes, 16));
    } else if (L.inter.npp > 0) {
        // pair search: cells of at least the cutoff, hashed into >= 2 buckets per vertex
        PairGrid& G = L.pgrid;
        const int N[3] = {L.d.nx, L.d.ny, L.d.nz};
        for (int a = 0; a < 3; ++a) {
            G.nc[a] = std::max(1, (int)std::floor((double)N[a] / L.inter.pp_cut));
            G.cs[a] = (double)N[a] / (double)G.nc[a];
        }
        G.table = 1024;
        while (G.table < 2u * (unsigned)L.nvert && G.table < (1u << 24)) G.table <<= 1;
        G.bits = 0;
        while ((1u << G.bits) < G.table) ++G.bits;
        for (int k = 0; k < 2; ++k) {
            BIB_ALLOC(c, (void**)&G.keys[k], L.nvert * sizeof(uint32_t));
            BIB_ALLOC(c, (void**)&G.ids[k], L.nvert * sizeof(uint32_t));
        }
        BIB_CUDA(c, cudaMemset(G.keys[1], 0, L.nvert * sizeof(uint32_t)));
        BIB_ALLOC(c, (void**)&G.start, G.table * sizeof(int));
        BIB_ALLOC(c, (void**)&G.end, G.table * sizeof(int));
        BIB_CUDA(c, cudaMemset(G.start, 0, G.table * sizeof(int)));
        BIB_CUDA(c, cudaMemset(G.end, 0, G.table * sizeof(int)));
        G.temp_bytes = pp_sort_temp_bytes(L.nvert, G.bits);
        BIB_ALLOC(c, &G.temp, std::max<size_t>(G.temp_bytes, 16));
    }
    if (L.phase) {
        // the reference voxelizes the membranes into the phase field when the immersed-boundary
        // functional first runs (ImmersedBoundaryDynamics.hh:404-412) and after every move
        const int64_t ncol = (int64_t)L.d.nx * L.d.ny;
        BIB_ALLOC(c, (void**)&L.vox_count, ncol * sizeof(int));
        BIB_CUDA(c, cudaMemset(L.vox_count, 0, ncol * sizeof(int)));
        BIB_ALLOC(c, (void**)&L.vox_z, ncol * kVoxelCap * sizeof(double));
        launch_voxelize(L, L.pos[L.pcur], c->stream);
    }
    BIB_CHECK_LAUNCH(c);
    L.particles_dirty = false;
    drop_graphs(c, L.handle);
    return BIB_OK;
}

// Phase boundaries of a step.  With profiling on: an event on the stream for the per-phase device
// times, and an NVTX range per phase named after the reference's Profile timers
// (fsi/Profile.h:26-97; the drivers time "compute_forces", "spread_forces", "lbm" around
// collideAndStream and its wall processors, "interpolate" and "move") for nsys / ncu timelines.
void record(bib_ctx* c, int idx) {
    if (!c->profiling) return;
    cudaEventRecord(c->ev[idx], c->stream);
    static const char* const kPhase[5] = {"compute_forces", "spread_forces", "lbm", "lbm (wall processors)",
                                          "interpolate + move"};
    if (idx > 0) nvtxRangePop();
    if (idx < 5) nvtxRangePushA(kPhase[idx]);
}


// One coupled step.  The reference's driver order (progs/capsule_in_shear/capsule_in_shear.cpp:
// 187-227) is computeVelocity -> setExternalVector -> [interpolate, compute + spread forces,
// move] -> collideAndStream -> wall processors.  Forces at X_n do not depend on the velocity,
// so the same arithmetic is issued as: membrane forces at X_n -> spreading into the force
// buffer that the previous step reset to the body force -> collide-and-stream, which also
// emits the velocity field of the pre-collision state with the previous force -> wall
// reconstruction -> interpolation of that velocity to X_n and the move -> area / volume /
// centre of the new positions.
//
// With a phase field and particles the collision needs the phase of the moved membranes
// (move_vertices_and_revoxelize, ImmersedBoundaryDynamics.hh:461-483, runs before
// collideAndStream), so the move comes first: velocity field of the current state ->
// interpolation and move -> area / volume / centre -> voxelization -> collide-and-stream.
void enqueue_step(bib_ctx* c, Lattice& L, bool with_ib, bool with_lbm) {
    cudaStream_t s = c->stream;
    const bool ib = with_ib && L.nvert > 0;
    if (with_ib && with_lbm && ib && L.phase) {
        if (!L.target_clean) launch_force_fill(L, 1 - L.fe, s);
        record(c, 0);
        launch_membrane_forces(L, s);
        launch_pp_forces(L, s);
        record(c, 1);
        launch_spread(L, 1 - L.fe, s);
        record(c, 2);
        launch_velocity_field(L, s);
        launch_interpolate_move(L, s);
        launch_particle_update(L, s);
        L.pcur = 1 - L.pcur;
        launch_voxelize(L, L.pos[L.pcur], s);
        launch_collide_stream(L, Coupling::kDense, s);
        forces_touched(L);
        record(c, 3);
        L.cur = 1 - L.cur;
        L.fe = 1 - L.fe;
        L.target_clean = true;
        launch_fd_walls(L, L.cur, L.fe, s);
        record(c, 4);
        record(c, 5);
        return;
    }
    if (with_ib && with_lbm) {
        // Sparse coupling: the collision reads only the force spread in this step and writes
        // the velocity field j/rho + body/2; the interpolation adds the previous force's share
        // (F[fe] - body)/2 at its support nodes; then F[fe] is reset to the body force at the
        // nodes its spreading recorded (or everywhere, when those are not known).
        const bool sparse = ib && sparse_coupling(L);
        if (!L.target_clean) launch_force_fill(L, 1 - L.fe, s);
        record(c, 0);
        if (ib) launch_membrane_forces(L, s);
        if (ib) launch_pp_forces(L, s);
        record(c, 1);
        if (ib) launch_spread(L, 1 - L.fe, s, sparse);
        if (sparse) L.sparse_ok[1 - L.fe] = true;  // a clean target plus the recorded nodes
        else forces_touched(L);
        record(c, 2);
        // dense: u of this state, collision with F[1-fe], F[fe] := body
        launch_collide_stream(L, sparse ? Coupling::kSparse : Coupling::kDense, s);
        record(c, 3);
        L.cur = 1 - L.cur;
        L.fe = 1 - L.fe;
        L.target_clean = !sparse;
        launch_fd_walls(L, L.cur, L.fe, s);
        record(c, 4);
        if (ib) {
            launch_interpolate_move(L, s, sparse ? 1 - L.fe : -1);
            if (sparse) {
                if (L.sparse_ok[1 - L.fe]) launch_force_clear(L, 1 - L.fe, s);
                else launch_force_fill(L, 1 - L.fe, s);
                L.sparse_ok[1 - L.fe] = true;  // all body force now
                L.target_clean = true;
            }
            launch_particle_update(L, s);
            L.pcur = 1 - L.pcur;
        }
        record(c, 5);
        return;
    }
    if (with_ib) {
        // the IB data processor alone: velocity of the current state, force field reset to
        // the body force, forces, spreading, move (DataProcessors.hh:104-107)
        record(c, 0);
        launch_velocity_field(L, s);
        launch_force_fill(L, L.fe, s);
        L.target_clean = false;
        forces_touched(L);
        if (ib) launch_membrane_forces(L, s);
        if (ib) launch_pp_forces(L, s);
        record(c, 1);
        if (ib) launch_spread(L, L.fe, s);
        record(c, 2);
        record(c, 3);
        record(c, 4);
        if (ib) {
            launch_interpolate_move(L, s);
            launch_particle_update(L, s);
            L.pcur = 1 - L.pcur;
            launch_voxelize(L, L.pos[L.pcur], s);
        }
        record(c, 5);
        return;
    }
    // collide-and-stream alone (CoProcessor3D::collideAndStream): collision with the current
    // external force, which stays as it is
    record(c, 0);
    record(c, 1);
    record(c, 2);
    launch_collide_stream(L, Coupling::kNone, s);
    record(c, 3);
    L.cur = 1 - L.cur;
    launch_fd_walls(L, L.cur, L.fe, s);
    record(c, 4);
    record(c, 5);
}

bib_status accumulate_profile(bib_ctx* c) {
    if (!c->profiling) return BIB_OK;
    BIB_CUDA(c, cudaEventSynchronize(c->ev[5]));
    for (int k = 0; k < 5; ++k) {
        float ms = 0;
        BIB_CUDA(c, cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]));
        c->prof[k] += ms;
    }
    return BIB_OK;
}

// The instantiated graph of `steps` (1 or 2) coupled steps from the lattice's current parity
// state, captured on first use.  Capturing leaves the host-side state as it was.
bib_status step_graph(bib_ctx* c, Lattice& L, int steps, cudaGraphExec_t* out) {
    // the captured launches depend on the parities and, for the sparse coupling, on whether
    // the previous force field can be reset at its recorded nodes
    const int sparse_key = sparse_coupling(L) ? 1 + (L.sparse_ok[L.fe] ? 1 : 0) : 0;
    const std::pair<int, int> key(L.handle, sparse_key * 16 + (steps - 1) * 8 + L.cur * 4 + L.pcur * 2 + L.fe);
    GraphEntry& ge = c->graphs[key];
    if (!ge.exec) {
        const int cur0 = L.cur, pcur0 = L.pcur, fe0 = L.fe;
        const bool clean0 = L.target_clean, ok0 = L.sparse_ok[0], ok1 = L.sparse_ok[1];
        cudaGraph_t g = nullptr;
        BIB_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < steps; ++k) enqueue_step(c, L, true, true);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        L.cur = cur0;
        L.pcur = pcur0;
        L.fe = fe0;
        L.target_clean = clean0;
        L.sparse_ok[0] = ok0;
        L.sparse_ok[1] = ok1;
        if (e != cudaSuccess) return fail(c, BIB_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
        size_t nn = 0;
        if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn) {
            std::vector<cudaGraphNode_t> nodes(nn);
            if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess) {
                ge.kernels = 0;
                for (size_t k = 0; k < nn; ++k) {
                    cudaGraphNodeType t;
                    if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++ge.kernels;
                }
            }
        }
        e = cudaGraphInstantiate(&ge.exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            ge.exec = nullptr;
            return fail(c, BIB_ECUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
        }
    }
    *out = ge.exec;
    return BIB_OK;
}

bib_status run_steps(bib_ctx* c, int32_t h, int64_t nsteps, bool with_ib, bool with_lbm) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle %d", h);
    if (nsteps < 0) return fail(c, BIB_EINVAL, "negative step count");
    bib_status st = sync_particles(c, *L);
    if (st) return st;
    const bool use_graph = c->graph_mode && !c->profiling && with_ib && with_lbm && nsteps >= 1;
    int64_t done = 0;
    if (use_graph) {
        // the graphs assume a clean spreading target on entry (and, for the sparse coupling, a
        // previous force field with known nodes, which one eager step establishes)
        if (!L->target_clean || (sparse_coupling(*L) && !L->sparse_ok[L->fe])) {
            enqueue_step(c, *L, true, true);
            BIB_CHECK_LAUNCH(c);
            ++done;
        }
        // a two-step graph leaves every parity unchanged; a one-step graph (the step-then-read
        // loop) exists per parity state and flips all three
        if (done + 2 <= nsteps) {
            cudaGraphExec_t g2 = nullptr;
            st = step_graph(c, *L, 2, &g2);
            if (st) return st;
            for (; done + 2 <= nsteps; done += 2) BIB_CUDA(c, cudaGraphLaunch(g2, c->stream));
        }
        if (done < nsteps) {
            cudaGraphExec_t g1 = nullptr;
            st = step_graph(c, *L, 1, &g1);
            if (st) return st;
            BIB_CUDA(c, cudaGraphLaunch(g1, c->stream));
            L->cur = 1 - L->cur;
            L->pcur = 1 - L->pcur;
            L->fe = 1 - L->fe;
            ++done;
        }
    }
    for (; done < nsteps; ++done) {
        enqueue_step(c, *L, with_ib, with_lbm);
        BIB_CHECK_LAUNCH(c);
        if (c->profiling) {
            st = accumulate_profile(c);
            if (st) return st;
        }
    }
    BIB_CHECK_LAUNCH(c);
    L->iteration += (uint64_t)nsteps;
    return BIB_OK;
}

// Make the host copies of the particle state authoritative again (before they change).
bib_status pull_particles(bib_ctx* c, Lattice& L) {
    if (L.particles_dirty || L.nvert == 0) return BIB_OK;
    L.host_pos.assign(3 * (size_t)L.nvert, 0.0);
    L.host_stats.assign(STATS * L.parts.size(), 0.0);
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    BIB_CUDA(c, cudaMemcpy(L.host_pos.data(), L.pos[L.pcur], L.host_pos.size() * 8, cudaMemcpyDeviceToHost));
    BIB_CUDA(c, cudaMemcpy(L.host_stats.data(), L.stats, L.host_stats.size() * 8, cudaMemcpyDeviceToHost));
    return BIB_OK;
}

// ---- host <-> device population transfers (bib_lattice_send / _receive)
//
// Page-locked host buffers (cudaHostAlloc, cudaMallocHost, cudaHostRegister: with unified
// addressing the device reaches them at an address it is told by cudaPointerGetAttributes) are
// read and written by the import / export kernels themselves, in one pass over the lattice that
// streams over the CPU-GPU link.  Pageable buffers go through two device staging halves: the
// copies of one chunk run on a copy stream while the kernel converts the other chunk.
//
// A transfer in wire order: structure of arrays (19 arrays of n doubles, x fastest; chunks of
// z-planes) or cell-major (`per` doubles per cell, z fastest and x slowest; chunks of x-planes).
struct Wire {
    int per;   // 0: structure of arrays; 19 or 23: doubles per cell, cell-major
};

// Device address of the host range [p, p + bytes) if the device can access it directly
// (page-locked memory mapped into the unified address space, both ends of one mapping), else null.
const void* device_view_of_host(const void* p, size_t bytes) {
    if (!p || bytes == 0) return nullptr;
    cudaPointerAttributes a{}, b{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    const char* last = static_cast<const char*>(p) + (bytes - 1);
    if (cudaPointerGetAttributes(&b, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (b.type != cudaMemoryTypeHost || !b.devicePointer) return nullptr;
    if (static_cast<const char*>(b.devicePointer) - static_cast<const char*>(a.devicePointer) != (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a.devicePointer;
}

// Staging halves of at least one chunk unit (a z-plane of 19 populations, or an x-plane of
// cells) and about 32 MB each; the copy stream and its events are made on first use.
constexpr size_t kStageHalf = (size_t)4 << 20;  // doubles

bib_status transfer_setup(bib_ctx* c, size_t unit, int64_t units, int64_t* per_chunk) {
    if (!c->copy_stream) {
        BIB_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            BIB_CUDA(c, cudaEventCreateWithFlags(&c->tx_ready[k], cudaEventDisableTiming));
            BIB_CUDA(c, cudaEventCreateWithFlags(&c->tx_free[k], cudaEventDisableTiming));
        }
        BIB_CUDA(c, cudaEventCreateWithFlags(&c->tx_start, cudaEventDisableTiming));
    }
    const size_t half = unit * std::max<size_t>(1, std::min<size_t>(kStageHalf / unit, (size_t)units));
    if (c->stage_count < 2 * half) {
        BIB_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(c->stage);
        c->stage = nullptr;
        c->stage_count = 0;
        BIB_ALLOC(c, (void**)&c->stage, 2 * half * sizeof(double));
        c->stage_count = 2 * half;
    }
    *per_chunk = (int64_t)std::min<size_t>(c->stage_count / 2 / unit, (size_t)units);
    return BIB_OK;
}

// Host populations in wire order -> lattice state (for the Palabos order also the force and
// the phase), in stream order; returns once the host buffer has been read.
bib_status import_populations(bib_ctx* c, Lattice& L, const double* src, Wire w) {
    const LatticeDesc& d = L.d;
    const int64_t n = d.n, plane = (int64_t)d.nx * d.ny, xplane = (int64_t)d.ny * d.nz;
    const size_t bytes = (size_t)(w.per ? w.per : Q) * n * sizeof(double);
    if (const double* m = static_cast<const double*>(device_view_of_host(src, bytes))) {
        if (w.per) launch_import_aos(L, m, w.per, 0, n, c->stream);
        else launch_import_planes(L, m, 0, d.nz, n, c->stream);
        BIB_CHECK_LAUNCH(c);
        BIB_CUDA(c, cudaStreamSynchronize(c->stream));
        return BIB_OK;
    }
    int64_t P = 0;
    const size_t unit = w.per ? (size_t)w.per * xplane : (size_t)Q * plane;
    bib_status st = transfer_setup(c, unit, w.per ? d.nx : d.nz, &P);
    if (st) return st;
    const size_t half = c->stage_count / 2;
    // the copies must not overtake earlier work of the main stream on the staging area
    BIB_CUDA(c, cudaEventRecord(c->tx_start, c->stream));
    BIB_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->tx_start, 0));
    const int64_t total = w.per ? d.nx : d.nz;
    int k = 0;
    for (int64_t a = 0; a < total; a += P, ++k) {
        const int64_t cnt = std::min<int64_t>(P, total - a);
        double* buf = c->stage + (size_t)(k & 1) * half;
        if (k >= 2) BIB_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->tx_free[k & 1], 0));
        if (w.per) {
            BIB_CUDA(c, cudaMemcpyAsync(buf, src + (size_t)w.per * a * xplane, (size_t)w.per * cnt * xplane * sizeof(double),
                                        cudaMemcpyHostToDevice, c->copy_stream));
        } else {
            const int64_t cc = plane * cnt;
            for (int i = 0; i < Q; ++i)
                BIB_CUDA(c, cudaMemcpyAsync(buf + i * cc, src + i * n + a * plane, cc * sizeof(double),
                                            cudaMemcpyHostToDevice, c->copy_stream));
        }
        BIB_CUDA(c, cudaEventRecord(c->tx_ready[k & 1], c->copy_stream));
        BIB_CUDA(c, cudaStreamWaitEvent(c->stream, c->tx_ready[k & 1], 0));
        if (w.per) launch_import_aos(L, buf, w.per, a * xplane, cnt * xplane, c->stream);
        else launch_import_planes(L, buf, (int)a, (int)cnt, plane * cnt, c->stream);
        BIB_CHECK_LAUNCH(c);
        BIB_CUDA(c, cudaEventRecord(c->tx_free[k & 1], c->stream));
    }
    BIB_CUDA(c, cudaStreamSynchronize(c->copy_stream));
    return BIB_OK;
}

// Lattice state -> host populations in wire order (Palabos order: with the force and the
// phase); returns once the host buffer holds them.
bib_status export_populations(bib_ctx* c, Lattice& L, double* dst, Wire w) {
    const LatticeDesc& d = L.d;
    const int64_t n = d.n, plane = (int64_t)d.nx * d.ny, xplane = (int64_t)d.ny * d.nz;
    const size_t bytes = (size_t)(w.per ? w.per : Q) * n * sizeof(double);
    if (double* m = static_cast<double*>(const_cast<void*>(device_view_of_host(dst, bytes)))) {
        if (w.per) launch_export_aos(L, m, w.per, 0, n, c->stream);
        else launch_export_planes(L, m, 0, d.nz, n, c->stream);
        BIB_CHECK_LAUNCH(c);
        BIB_CUDA(c, cudaStreamSynchronize(c->stream));
        return BIB_OK;
    }
    int64_t P = 0;
    const size_t unit = w.per ? (size_t)w.per * xplane : (size_t)Q * plane;
    bib_status st = transfer_setup(c, unit, w.per ? d.nx : d.nz, &P);
    if (st) return st;
    const size_t half = c->stage_count / 2;
    const int64_t total = w.per ? d.nx : d.nz;
    const int nchunks = (int)((total + P - 1) / P);
    auto convert = [&](int k) -> bib_status {
        const int64_t a = (int64_t)k * P, cnt = std::min<int64_t>(P, total - a);
        double* buf = c->stage + (size_t)(k & 1) * half;
        if (k >= 2) BIB_CUDA(c, cudaStreamWaitEvent(c->stream, c->tx_free[k & 1], 0));
        if (w.per) launch_export_aos(L, buf, w.per, a * xplane, cnt * xplane, c->stream);
        else launch_export_planes(L, buf, (int)a, (int)cnt, plane * cnt, c->stream);
        BIB_CHECK_LAUNCH(c);
        BIB_CUDA(c, cudaEventRecord(c->tx_ready[k & 1], c->stream));
        return BIB_OK;
    };
    // the kernel of chunk k + 1 is queued before the copies of chunk k: a copy into pageable
    // memory returns only when it is done, and the kernel runs meanwhile
    st = convert(0);
    if (st) return st;
    for (int k = 0; k < nchunks; ++k) {
        if (k + 1 < nchunks) {
            st = convert(k + 1);
            if (st) return st;
        }
        const int64_t a = (int64_t)k * P, cnt = std::min<int64_t>(P, total - a);
        const double* buf = c->stage + (size_t)(k & 1) * half;
        BIB_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->tx_ready[k & 1], 0));
        if (w.per) {
            BIB_CUDA(c, cudaMemcpyAsync(dst + (size_t)w.per * a * xplane, buf, (size_t)w.per * cnt * xplane * sizeof(double),
                                        cudaMemcpyDeviceToHost, c->copy_stream));
        } else {
            const int64_t cc = plane * cnt;
            for (int i = 0; i < Q; ++i)
                BIB_CUDA(c, cudaMemcpyAsync(dst + i * n + a * plane, buf + i * cc, cc * sizeof(double),
                                            cudaMemcpyDeviceToHost, c->copy_stream));
        }
        BIB_CUDA(c, cudaEventRecord(c->tx_free[k & 1], c->copy_stream));
    }
    BIB_CUDA(c, cudaStreamSynchronize(c->copy_stream));
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    return BIB_OK;
}

bib_status device_buffer(bib_ctx* c, double** d, const double* host, size_t count) {
    BIB_ALLOC(c, (void**)d, count * sizeof(double));
    if (host) BIB_CUDA(c, cudaMemcpyAsync(*d, host, count * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return BIB_OK;
}

}  // namespace

// =================================================================== batches
// A batch steps several lattices in lockstep with one launch per kernel for all of them.
// Its device tables hold, for each of the two step parities, one IbView and one CollideView
// per lattice; the lattices' own parities (cur, fe, pcur) advance together.
struct Batch {
    std::vector<int32_t> handles;
    int storage = 0, collision = 0, dirac = 0;
    IbView* views[2] = {nullptr, nullptr};
    CollideView* cviews[2] = {nullptr, nullptr};
    ParticleDev* parts = nullptr;
    int* vinst = nullptr;
    int nparts = 0, nvert = 0, max_nv = 0;
    size_t membrane_smem = 0;
    int64_t ntiles = 0;
    int any_fd = 0, nx_max = 0, nz_max = 0;
    int any_phase = 0;                  // a lattice voxelizes its particles into a phase field
    int tile_cells = 0, stages = 0, membrane_block = 256;
    int phase = 0;                      // parity of the next step relative to the tables
    std::vector<uint64_t> versions;     // lattice versions the tables were built for
    std::vector<int> state0;            // per lattice: cur*4 + pcur*2 + fe at phase 0
    bool built = false;
    GraphEntry graph[2];
    void free_tables() {
        for (int p = 0; p < 2; ++p) {
            cudaFree(views[p]);
            cudaFree(cviews[p]);
            views[p] = nullptr;
            cviews[p] = nullptr;
            if (graph[p].exec) cudaGraphExecDestroy(graph[p].exec);
            graph[p].exec = nullptr;
        }
        cudaFree(parts);
        cudaFree(vinst);
        parts = nullptr;
        vinst = nullptr;
        built = false;
    }
    ~Batch() { free_tables(); }
};

bib_ctx::~bib_ctx() = default;

namespace {

Batch* get_batch(bib_ctx* c, int32_t b) {
    if (!c || b < 0 || b >= (int32_t)c->batches.size()) return nullptr;
    return c->batches[b].get();
}

int lattice_state(const Lattice& L) { return L.cur * 4 + L.pcur * 2 + L.fe; }

// (Re)build the device tables from the lattices' current state, which becomes phase 0.
bib_status build_batch(bib_ctx* c, Batch& B) {
    B.free_tables();
    const int n = (int)B.handles.size();
    std::vector<IbView> iv[2];
    std::vector<CollideView> cv[2];
    std::vector<ParticleDev> parts;
    std::vector<int> vinst;
    B.versions.assign(n, 0);
    B.state0.assign(n, 0);
    B.max_nv = 0;
    B.ntiles = 0;
    B.any_fd = 0;
    B.any_phase = 0;
    B.nx_max = B.nz_max = 0;
    int vbase = 0;
    for (int i = 0; i < n; ++i) {
        Lattice& L = *get_lattice(c, B.handles[i]);
        bib_status st = sync_particles(c, L);
        if (st) return st;
        if (L.inter.npp > 0)
            return fail(c, BIB_EUNSUPPORTED, "batched steps do not evaluate particle-particle interactions (lattice %d)",
                        B.handles[i]);
        if (L.nguo > 0)
            return fail(c, BIB_EUNSUPPORTED, "batched steps do not apply second-order rigid walls (lattice %d)",
                        B.handles[i]);
        B.versions[i] = L.version;
        B.state0[i] = lattice_state(L);
        for (int p = 0; p < 2; ++p) {
            // phase p: every parity of the lattice flipped p times
            const int cur = L.cur ^ p, fe = L.fe ^ p, pcur = L.nvert ? (L.pcur ^ p) : L.pcur;
            IbView v{};
            v.d = L.d;
            v.ib = L.ib;
            v.pos = L.pos[pcur];
            v.pos_next = L.pos[1 - pcur];
            v.u = L.u;
            v.vel = L.vel;
            v.force = L.force;
            v.F = L.F[1 - fe];
            v.stats = L.stats;
            v.vbase = vbase;
            v.nvert = L.nvert;
            iv[p].push_back(v);
            CollideView w{};
            if (!staged_collide_view(L, B.tile_cells, w))
                return fail(c, BIB_EUNSUPPORTED, "lattice %d does not fit the staged collide-and-stream kernel", B.handles[i]);
            w.fin = L.f[cur];
            w.fout = L.f[1 - cur];
            w.wall = L.wall;
            w.Fcol = L.F[1 - fe];
            w.Fprev = L.F[fe];
            w.u = L.u;
            w.phase = L.phase;
            w.celltype = L.celltype;
            w.tile0 = B.ntiles;
            cv[p].push_back(w);
        }
        B.ntiles += cv[0].back().ntiles;
        B.any_fd |= L.d.fd_walls;
        B.any_phase |= (L.phase && L.nvert) ? 1 : 0;
        B.nx_max = std::max(B.nx_max, L.d.nx);
        B.nz_max = std::max(B.nz_max, L.d.nz);
        for (size_t k = 0; k < L.pdev_host.size(); ++k) {
            ParticleDev d = L.pdev_host[k];
            d.inst = i;
            parts.push_back(d);
        }
        for (int v = 0; v < L.nvert; ++v) vinst.push_back(i);
        vbase += L.nvert;
        B.max_nv = std::max(B.max_nv, L.max_nv);
    }
    B.nparts = (int)parts.size();
    B.nvert = vbase;
    B.membrane_smem = membrane_smem_bytes(B.max_nv);
    configure_membrane_kernel(B.membrane_smem);
    bib_status st;
    for (int p = 0; p < 2; ++p)
        if ((st = upload(c, &B.views[p], iv[p])) || (st = upload(c, &B.cviews[p], cv[p]))) return st;
    if ((st = upload(c, &B.parts, parts)) || (st = upload(c, &B.vinst, vinst))) return st;
    B.phase = 0;
    B.built = true;
    return BIB_OK;
}

// Bring the tables up to date with the lattices; returns the phase of the next step.
bib_status prepare_batch(bib_ctx* c, Batch& B) {
    bool rebuild = !B.built;
    const int n = (int)B.handles.size();
    for (int i = 0; i < n && !rebuild; ++i) {
        Lattice* L = get_lattice(c, B.handles[i]);
        if (!L) return fail(c, BIB_EINVAL, "a lattice of the batch has been destroyed");
        if (L->particles_dirty || L->version != B.versions[i]) rebuild = true;
    }
    if (!rebuild) {  // every lattice must sit at the batch's phase
        for (int i = 0; i < n && !rebuild; ++i) {
            const Lattice& L = *get_lattice(c, B.handles[i]);
            const int s0 = B.state0[i];
            const int want = B.phase ? (s0 ^ (L.nvert ? 7 : 5)) : s0;
            if (lattice_state(L) != want) rebuild = true;
        }
    }
    if (rebuild) {
        bib_status st = build_batch(c, B);
        if (st) return st;
    }
    // the coupled step expects every spreading target already reset to the body force
    for (int i = 0; i < n; ++i) {
        Lattice& L = *get_lattice(c, B.handles[i]);
        if (!L.target_clean) {
            launch_force_fill(L, 1 - L.fe, c->stream);
            L.target_clean = true;
        }
    }
    BIB_CHECK_LAUNCH(c);
    return BIB_OK;
}

BatchLaunch batch_launch(bib_ctx* c, const Batch& B, int phase) {
    BatchLaunch bl;
    bl.n = (int)B.handles.size();
    bl.storage = B.storage;
    bl.collision = B.collision;
    bl.dirac = B.dirac;
    bl.views = B.views[phase];
    bl.cviews = B.cviews[phase];
    bl.wviews = B.cviews[phase ^ 1];
    bl.parts = B.parts;
    bl.nparts = B.nparts;
    bl.vinst = B.vinst;
    bl.nvert = B.nvert;
    bl.max_nv = B.max_nv;
    bl.membrane_smem = B.membrane_smem;
    bl.ntiles = B.ntiles;
    bl.stages = B.stages;
    bl.any_fd = B.any_fd;
    bl.nx_max = B.nx_max;
    bl.nz_max = B.nz_max;
    bl.wait_err = c->d_flag + 1;
    return bl;
}

// One coupled step of every lattice of the batch (the order of enqueue_step).  With a phase field
// the collision needs the phase of the moved membranes: the move comes first (velocity field of
// the current state per lattice, interpolation and move, update, voxelization per lattice of the
// moved membranes), then collide-and-stream.  The interpolated velocity is the same either way.
bib_status enqueue_batch_step(bib_ctx* c, Batch& B) {
    const BatchLaunch bl = batch_launch(c, B, B.phase);
    launch_membrane_batch(bl, B.membrane_block, c->stream);
    launch_spread_batch(bl, c->stream);
    if (B.any_phase) {
        for (int32_t h : B.handles) {
            Lattice& L = *get_lattice(c, h);
            if (L.nvert) launch_velocity_field(L, c->stream);
        }
        launch_interpolate_batch(bl, c->stream);
        launch_update_batch(bl, c->stream);
        for (int32_t h : B.handles) {
            Lattice& L = *get_lattice(c, h);
            if (L.phase && L.nvert) launch_voxelize(L, L.pos[1 - L.pcur], c->stream);
        }
        if (!launch_collide_batch(bl, c->stream))
            return fail(c, BIB_EUNSUPPORTED, "batched collide-and-stream could not be launched (shared memory)");
        launch_fd_walls_batch(bl, c->stream);
    } else {
        if (!launch_collide_batch(bl, c->stream))
            return fail(c, BIB_EUNSUPPORTED, "batched collide-and-stream could not be launched (shared memory)");
        launch_fd_walls_batch(bl, c->stream);
        launch_interpolate_batch(bl, c->stream);
        launch_update_batch(bl, c->stream);
    }
    for (int32_t h : B.handles) {
        Lattice& L = *get_lattice(c, h);
        L.cur ^= 1;
        L.fe ^= 1;
        if (L.nvert) L.pcur ^= 1;
        L.target_clean = true;
        forces_touched(L);
    }
    B.phase ^= 1;
    return BIB_OK;
}

bib_status run_batch(bib_ctx* c, Batch& B, int64_t nsteps) {
    bib_status st = prepare_batch(c, B);
    if (st) return st;
    int64_t done = 0;
    if (c->graph_mode && nsteps >= 2) {
        GraphEntry& ge = B.graph[B.phase];
        if (!ge.exec) {
            std::vector<int> saved;
            for (int32_t h : B.handles) saved.push_back(lattice_state(*get_lattice(c, h)));
            const int phase0 = B.phase;
            cudaGraph_t g = nullptr;
            BIB_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            bib_status s1 = enqueue_batch_step(c, B);
            bib_status s2 = s1 ? s1 : enqueue_batch_step(c, B);
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            for (size_t i = 0; i < B.handles.size(); ++i) {  // two steps: every parity back where it was
                Lattice& L = *get_lattice(c, B.handles[i]);
                L.cur = saved[i] >> 2;
                L.pcur = (saved[i] >> 1) & 1;
                L.fe = saved[i] & 1;
            }
            B.phase = phase0;
            if (s2) {
                if (g) cudaGraphDestroy(g);
                return s2;
            }
            if (e != cudaSuccess) return fail(c, BIB_ECUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&ge.exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(c, BIB_ECUDA, "batch graph instantiation failed: %s", cudaGetErrorString(e));
        }
        for (; done + 2 <= nsteps; done += 2) BIB_CUDA(c, cudaGraphLaunch(ge.exec, c->stream));
    }
    for (; done < nsteps; ++done) {
        st = enqueue_batch_step(c, B);
        if (st) return st;
        BIB_CHECK_LAUNCH(c);
    }
    BIB_CHECK_LAUNCH(c);
    for (int32_t h : B.handles) get_lattice(c, h)->iteration += (uint64_t)nsteps;
    return BIB_OK;
}

bib_status timed(bib_ctx* c, const std::function<bib_status()>& fn, double* ms) {
    cudaEvent_t a, b;
    BIB_CUDA(c, cudaEventCreate(&a));
    BIB_CUDA(c, cudaEventCreate(&b));
    BIB_CUDA(c, cudaEventRecord(a, c->stream));
    bib_status st = fn();
    BIB_CUDA(c, cudaEventRecord(b, c->stream));
    BIB_CUDA(c, cudaEventSynchronize(b));
    float f = 0;
    BIB_CUDA(c, cudaEventElapsedTime(&f, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = f;
    return st;
}

}  // namespace

// =================================================================== C ABI
extern "C" {

int32_t bib_abi_version(void) { return BIB_ABI_VERSION; }

const char* bib_status_string(bib_status s) {
    switch (s) {
        case BIB_OK: return "ok";
        case BIB_EINVAL: return "invalid argument";
        case BIB_ENOMEM: return "out of memory";
        case BIB_ECUDA: return "CUDA error";
        case BIB_ENAN: return "NaN or Inf in the state";
        case BIB_ETIMEOUT: return "device wait timed out";
        case BIB_ESTATE: return "invalid call order";
        case BIB_EUNSUPPORTED: return "unsupported option";
        case BIB_EOVERFLOW: return "device buffer overflow";
        default: return "unknown status";
    }
}

bib_status bib_create(const bib_config* cfg, bib_ctx** out) {
    if (!out) return BIB_EINVAL;
    *out = nullptr;
    bib_ctx* c = new (std::nothrow) bib_ctx();
    if (!c) return BIB_ENOMEM;
    c->device = cfg ? cfg->device : 0;
    if (const char* fa = std::getenv("BIB_FAIL_DEVICE_ALLOC")) c->fail_alloc = std::atoll(fa);
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) e = cudaEventCreate(&c->ev[k]);
    for (int k = 0; k < 8 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&c->dl_ev[k], cudaEventDisableTiming);
    // d_flag[0]: NaN scan result, d_flag[1]: set by a bounded device wait that gave up,
    // d_flag[2]: set by a voxelization whose column held more crossings than it can store
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_flag, 3 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_flag, 0, 3 * sizeof(int));
    if (e != cudaSuccess) {
        delete c;
        return BIB_ECUDA;
    }
    // set-up of bib_spread_forces_noalloc: the static scratch array's address on this device
    std::string msg;
    if (spread_scratch_address(&c->spread_scratch, msg) != BIB_OK) {
        bib_destroy(c);
        return BIB_ECUDA;
    }
    *out = c;
    return BIB_OK;
}

void bib_destroy(bib_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& kv : c->graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    for (auto& Lp : c->lattices) {
        if (!Lp) continue;
        free_particles(*Lp);
        cudaFree(Lp->f[0]);
        cudaFree(Lp->f[1]);
        cudaFree(Lp->F[0]);
        cudaFree(Lp->F[1]);
        cudaFree(Lp->u);
        cudaFree(Lp->wall);
        cudaFree(Lp->phase);
        cudaFree(Lp->celltype);
        cudaFree(Lp->guo);
    }
    for (auto& S : c->shapes) {
        cudaFree(S->dev.rest);
        cudaFree(S->dev.tri);
        cudaFree(S->dev.tri_area);
        cudaFree(S->dev.links);
        cudaFree(S->dev.link_len);
        cudaFree(S->dev.pairs);
        cudaFree(S->dev.pair_cs);
        cudaFree(S->dev.inc_off);
        cudaFree(S->dev.inc);
        cudaFree(S->dev.tri_rest_f);
        cudaFree(S->dev.tri4);
        cudaFree(S->dev.tri_area_f);
        cudaFree(S->dev.pair_cs_f);
    }
    for (int k = 0; k < 6; ++k)
        if (c->ev[k]) cudaEventDestroy(c->ev[k]);
    for (int k = 0; k < 8; ++k)
        if (c->dl_ev[k]) cudaEventDestroy(c->dl_ev[k]);
    cudaFree(c->d_flag);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    cudaFree(c->stage);
    for (int k = 0; k < 2; ++k) {
        if (c->tx_ready[k]) cudaEventDestroy(c->tx_ready[k]);
        if (c->tx_free[k]) cudaEventDestroy(c->tx_free[k]);
    }
    if (c->tx_start) cudaEventDestroy(c->tx_start);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

bib_status bib_sync(bib_ctx* c) {
    if (!c) return BIB_EINVAL;
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    return BIB_OK;
}

size_t bib_last_error(const bib_ctx* c, char* buf, size_t len) {
    if (!c) return 0;
    if (buf && len) {
        std::strncpy(buf, c->err.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return c->err.size();
}

bib_status bib_set_graph_mode(bib_ctx* c, int32_t enabled) {
    if (!c) return BIB_EINVAL;
    c->graph_mode = enabled != 0;
    return BIB_OK;
}

bib_status bib_batch_create(bib_ctx* c, const int32_t* handles, int32_t n, int32_t* batch) {
    if (!c || !handles || n <= 0 || !batch) return fail(c, BIB_EINVAL, "null argument or empty batch");
    auto B = std::make_unique<Batch>();
    for (int32_t i = 0; i < n; ++i) {
        Lattice* L = get_lattice(c, handles[i]);
        if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle %d", handles[i]);
        for (int32_t j = 0; j < i; ++j)
            if (handles[j] == handles[i]) return fail(c, BIB_EINVAL, "lattice %d appears twice", handles[i]);
        if (i == 0) {
            B->storage = L->storage;
            B->collision = L->d.collision;
            B->dirac = L->ib.dirac;
        } else if (L->storage != B->storage || L->d.collision != B->collision || L->ib.dirac != B->dirac) {
            return fail(c, BIB_EINVAL, "the lattices of a batch share storage, collision and delta kernel");
        }
        if (L->ib.spread_mode != BIB_SPREAD_ATOMIC)
            return fail(c, BIB_EUNSUPPORTED, "batched steps spread with atomics (lattice %d is deterministic)", handles[i]);
        CollideView probe{};
        if (!staged_collide_view(*L, 0, probe))
            return fail(c, BIB_EUNSUPPORTED, "lattice %d does not fit the staged collide-and-stream kernel", handles[i]);
        B->handles.push_back(handles[i]);
    }
    *batch = (int32_t)c->batches.size();
    c->batches.push_back(std::move(B));
    return BIB_OK;
}

bib_status bib_batch_destroy(bib_ctx* c, int32_t b) {
    Batch* B = get_batch(c, b);
    if (!B) return fail(c, BIB_EINVAL, "invalid batch handle");
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    c->batches[b].reset();
    return BIB_OK;
}

bib_status bib_batch_step(bib_ctx* c, int32_t b, int64_t nsteps) {
    Batch* B = get_batch(c, b);
    if (!B) return fail(c, BIB_EINVAL, "invalid batch handle");
    if (nsteps < 0) return fail(c, BIB_EINVAL, "negative step count");
    return run_batch(c, *B, nsteps);
}

bib_status bib_batch_step_timed(bib_ctx* c, int32_t b, int64_t nsteps, double* ms) {
    Batch* B = get_batch(c, b);
    if (!B || !ms) return fail(c, BIB_EINVAL, "invalid batch handle or null argument");
    if (nsteps < 0) return fail(c, BIB_EINVAL, "negative step count");
    bib_status st = prepare_batch(c, *B);  // uploads happen outside the timed region
    if (st) return st;
    return timed(c, [&] { return run_batch(c, *B, nsteps); }, ms);
}

bib_status bib_batch_set_tuning(bib_ctx* c, int32_t b, const bib_batch_tuning* t) {
    Batch* B = get_batch(c, b);
    if (!B || !t) return fail(c, BIB_EINVAL, "invalid batch handle or tuning");
    if (t->tile_cells < 0 || t->stages < 0 || t->stages == 1 || t->stages > 4 ||
        (t->membrane_block != 0 && t->membrane_block != 64 && t->membrane_block != 128 && t->membrane_block != 256 &&
         t->membrane_block != 512))
        return fail(c, BIB_EINVAL, "invalid batch tuning values");
    if (!collide_batch_fits(B->storage, B->collision, t->stages))
        return fail(c, BIB_EUNSUPPORTED, "%d stages do not fit the shared memory of a CTA", t->stages);
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    B->tile_cells = t->tile_cells;
    B->stages = t->stages;
    B->membrane_block = t->membrane_block ? t->membrane_block : 256;
    B->free_tables();  // tile geometry and graphs depend on the tuning
    return BIB_OK;
}

bib_status bib_batch_autotune(bib_ctx* c, int32_t b, int32_t steps, bib_batch_tuning* chosen) {
    Batch* B = get_batch(c, b);
    if (!B || steps <= 0) return fail(c, BIB_EINVAL, "invalid batch handle or step count");
    // Every candidate runs `steps` real coupled steps (plain launches); the tile size, the
    // stage count and the membrane block size change the schedule, not the arithmetic.
    const int graph = c->graph_mode;
    c->graph_mode = false;
    bib_batch_tuning best{};
    double best_ms = 1e300;
    const int tiles[2] = {0, 256};
    for (int ti = 0; ti < 2; ++ti)
        for (int ns = 2; ns <= 4; ++ns) {
            bib_batch_tuning t{};
            t.tile_cells = tiles[ti];
            t.stages = ns;
            t.membrane_block = B->membrane_block;
            if (!collide_batch_fits(B->storage, B->collision, ns)) continue;
            bib_status st = bib_batch_set_tuning(c, b, &t);
            if (st) {
                c->graph_mode = graph;
                return st;
            }
            double ms = 0;
            st = bib_batch_step(c, b, 1);  // builds the tables outside the timed steps
            if (!st) st = bib_batch_step_timed(c, b, steps, &ms);
            if (st) {
                c->graph_mode = graph;
                return st;
            }
            if (ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
    double best_mb = 1e300;
    int best_block = 256;
    const int blocks[4] = {64, 128, 256, 512};
    for (int k = 0; k < 4; ++k) {
        bib_batch_tuning t = best;
        t.membrane_block = blocks[k];
        bib_status st = bib_batch_set_tuning(c, b, &t);
        double ms = 0;
        if (!st) st = bib_batch_step(c, b, 1);
        if (!st) st = bib_batch_step_timed(c, b, steps, &ms);
        if (st) {
            c->graph_mode = graph;
            return st;
        }
        if (ms < best_mb) {
            best_mb = ms;
            best_block = blocks[k];
        }
    }
    best.membrane_block = best_block;
    c->graph_mode = graph;
    bib_status st = bib_batch_set_tuning(c, b, &best);
    if (st) return st;
    if (chosen) *chosen = best;
    return BIB_OK;
}

bib_status bib_spread_forces_noalloc(bib_ctx* c, int32_t h, const double* pos, const double* force, int64_t nvert,
                                     void* field) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    std::string msg;
    const bib_status st = spread_noalloc(*L, c->device, c->spread_scratch, c->stream, pos, force, nvert, field, msg);
    if (st != BIB_OK) return fail(c, st, "%s", msg.c_str());
    return BIB_OK;
}

static bib_status set_cell_types_impl(bib_ctx* c, int32_t h, const uint8_t* types) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!types) {
        cudaFree(L->celltype);
        L->celltype = nullptr;
        L->d.has_types = 0;
    } else {
        for (int64_t k = 0; k < L->d.n; ++k)
            if (types[k] > BIB_CELL_NO_DYNAMICS) return fail(c, BIB_EINVAL, "cell type %d at cell %lld", (int)types[k], (long long)k);
        if (!L->celltype) BIB_ALLOC(c, (void**)&L->celltype, L->d.n);
        BIB_CUDA(c, cudaMemcpy(L->celltype, types, L->d.n, cudaMemcpyHostToDevice));
        L->d.has_types = 1;
    }
    drop_graphs(c, h);
    for (auto& B : c->batches)  // batch tables hold the lattice description
        if (B) B->free_tables();
    return BIB_OK;
}

bib_status bib_lattice_set_cell_types(bib_ctx* c, int32_t h, const uint8_t* types) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    // explicit cell types replace second-order pipe walls
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(L->guo);
    L->guo = nullptr;
    L->nguo = 0;
    return set_cell_types_impl(c, h, types);
}

// PipeBoundary::trace_ray (fsi/Boundary.h:164-187): crossing parameter t in [0, 1] of the
// segment p0 -> p1 with the cylinder of `radius` around the x axis through (y0, z0)
static bool pipe_trace_ray(double py0, double pz0, double radius, const double* p0, const double* p1, double& t) {
    const double y1 = p0[1] - py0, y2 = p1[1] - py0, z1 = p0[2] - pz0, z2 = p1[2] - pz0;
    const double a = (y2 - y1) * (y2 - y1) + (z2 - z1) * (z2 - z1);
    const double b = y1 * (y2 - y1) + z1 * (z2 - z1);
    const double c = y1 * y1 + z1 * z1 - radius * radius;
    const double disc = b * b - c * a;
    if (disc < 0. || std::fabs(a) < 10 * 2.220446049250313e-16) return false;
    const double bOverA = -b / a;
    const double sqrtDisc = std::sqrt(disc) / a;
    t = bOverA - sqrtDisc;
    if (t >= 0. && t <= 1.) return true;
    t = bOverA + sqrtDisc;
    return t >= 0. && t <= 1.;
}

bib_status bib_lattice_set_pipe_walls(bib_ctx* c, int32_t h, double y0, double z0, double radius, int32_t second_order) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    if (!(radius > 0) || !std::isfinite(y0) || !std::isfinite(z0) || second_order < 0 || second_order > 1)
        return fail(c, BIB_EINVAL, "bad pipe geometry");
    const int64_t nx = L->d.nx, ny = L->d.ny, nz = L->d.nz;
    std::vector<uint8_t> types((size_t)L->d.n);
    // PipeBoundary::contains (fsi/Boundary.h:149-152) with margins 0 and -(plint)sqrt(2)
    const double margin = -(double)(int64_t)std::sqrt(2.0);
    auto r2_of = [&](int64_t y, int64_t z) {
        const double dy = (double)y - y0, dz = (double)z - z0;
        return dy * dy + dz * dz;
    };
    for (int64_t z = 0; z < nz; ++z)
        for (int64_t y = 0; y < ny; ++y) {
            const double r2 = r2_of(y, z);
            uint8_t t = BIB_CELL_FLUID;
            if (!second_order && !(r2 < radius * radius)) t = BIB_CELL_BOUNCE_BACK;
            if (!(r2 < (radius - margin) * (radius - margin))) t = BIB_CELL_NO_DYNAMICS;
            std::fill(types.begin() + (size_t)(nx * (y + ny * z)), types.begin() + (size_t)(nx * (y + ny * z) + nx), t);
        }
    std::vector<GuoNode> nodes;
    if (second_order) {
        // GuoRigidWallBoundaryInstantiator::process (fsi/GuoBoundaryCondition.hh:62-130): nodes
        // outside the pipe with a lattice vector crossing the wall; among the crossing vectors the
        // one whose direction has the smallest cosine with the outward normal at the crossing
        static const int CX[Q] = {0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0};
        static const int CY[Q] = {0, 0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 1, 0, 1, -1, 0, 0, 1, 1};
        static const int CZ[Q] = {0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1};
        std::vector<int> is_wall((size_t)L->d.n, 0);
        for (int64_t x = 0; x < nx; ++x)
            for (int64_t y = 0; y < ny; ++y)
                for (int64_t z = 0; z < nz; ++z) {
                    const double pos[3] = {(double)x, (double)y, (double)z};
                    if (r2_of(y, z) < radius * radius) continue;
                    double cos_min = 2, delta_min = -1;
                    int dir_min = 0;
                    bool found = false;
                    for (int i = 1; i < Q; ++i) {
                        const double cv[3] = {(double)CX[i], (double)CY[i], (double)CZ[i]};
                        const double p2[3] = {pos[0] + cv[0], pos[1] + cv[1], pos[2] + cv[2]};
                        double t = -1;
                        if (!pipe_trace_ray(y0, z0, radius, pos, p2, t)) continue;
                        const double cn = std::sqrt((double)(CX[i] * CX[i] + CY[i] * CY[i] + CZ[i] * CZ[i]));
                        const double d2[3] = {cv[0] / cn, cv[1] / cn, cv[2] / cn};
                        const double w[3] = {pos[0] + d2[0] * t, pos[1] + d2[1] * t, pos[2] + d2[2] * t};
                        const double nv[3] = {0, w[1] - y0, w[2] - z0};  // PipeBoundary::get_normal
                        const double nn = std::sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
                        const double cosang = nv[0] / nn * d2[0] + nv[1] / nn * d2[1] + nv[2] / nn * d2[2];
                        if (cosang < cos_min) {
                            dir_min = i;
                            cos_min = cosang;
                            delta_min = 1 - t;
                        }
                        found = true;
                    }
                    if (!found) continue;
                    GuoNode g{};
                    g.x = (int)x, g.y = (int)y, g.z = (int)z;
                    g.dir = dir_min;
                    g.delta = delta_min;
                    g.nodyn = types[(size_t)(x + nx * (y + ny * z))] == BIB_CELL_NO_DYNAMICS;
                    nodes.push_back(g);
                    is_wall[(size_t)(x + nx * (y + ny * z))] = 1;
                }
        // the reconstruction reads two fluid nodes per wall node: they must be neither wall nodes nor
        // NoDynamics nodes (a pipe a few nodes wide would violate this)
        for (const GuoNode& g : nodes)
            for (int m = 1; m <= 2; ++m) {
                const int64_t xs = ((g.x + m * CX[g.dir]) % nx + nx) % nx, ys = ((g.y + m * CY[g.dir]) % ny + ny) % ny,
                              zs = ((g.z + m * CZ[g.dir]) % nz + nz) % nz;
                const size_t k = (size_t)(xs + nx * (ys + ny * zs));
                if (is_wall[k] || types[k] != BIB_CELL_FLUID)
                    return fail(c, BIB_EUNSUPPORTED, "pipe too narrow for the second-order walls");
            }
    }
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(L->guo);
    L->guo = nullptr;
    L->nguo = 0;
    if (!nodes.empty()) {
        BIB_ALLOC(c, (void**)&L->guo, nodes.size() * sizeof(GuoNode));
        BIB_CUDA(c, cudaMemcpy(L->guo, nodes.data(), nodes.size() * sizeof(GuoNode), cudaMemcpyHostToDevice));
        L->nguo = (int)nodes.size();
    }
    return set_cell_types_impl(c, h, types.data());
}

bib_status bib_lattice_set_tuning(bib_ctx* c, int32_t h, const bib_tuning* t) {
    Lattice* L = get_lattice(c, h);
    if (!L || !t) return fail(c, BIB_EINVAL, "invalid lattice handle or tuning");
    const int mb = t->membrane_block;
    if (t->collide_kernel < BIB_KERNEL_AUTO || t->collide_kernel > BIB_KERNEL_STAGED || t->tile_cells < 0 ||
        t->stages < 0 || t->stages == 1 || t->stages > 4 ||
        (mb != 0 && mb != 64 && mb != 128 && mb != 256 && mb != 512) ||
        (t->force_reset < BIB_FORCE_RESET_AUTO || t->force_reset > BIB_FORCE_RESET_SPARSE) || t->wait_limit_us < 0 ||
        t->withhold_tile < 0)
        return fail(c, BIB_EINVAL, "invalid tuning values");
    Lattice probe = {};
    probe.d = L->d;
    probe.storage = L->storage;
    probe.tile_cells = t->tile_cells;
    probe.stages = t->stages;
    if (t->collide_kernel == BIB_KERNEL_STAGED && !collide_staged_fits(probe))
        return fail(c, BIB_EUNSUPPORTED, "the staged collide-and-stream kernel does not fit this lattice / tile size");
    drop_graphs(c, h);
    L->collide_kernel = t->collide_kernel;
    L->tile_cells = t->tile_cells;
    L->stages = t->stages;
    L->membrane_block = mb ? mb : 256;
    L->sparse_reset = t->force_reset == BIB_FORCE_RESET_SPARSE;
    L->wait_ns = t->wait_limit_us ? (uint64_t)t->wait_limit_us * 1000u : kDefaultWaitNs;
    L->withhold_tile = (int64_t)t->withhold_tile - 1;
    forces_touched(*L);
    return BIB_OK;
}

bib_status bib_set_profiling(bib_ctx* c, int32_t enabled) {
    if (!c) return BIB_EINVAL;
    c->profiling = enabled != 0;
    for (double& v : c->prof) v = 0;
    return BIB_OK;
}

bib_status bib_profile_read(bib_ctx* c, double* out, int32_t n) {
    if (!c || !out) return BIB_EINVAL;
    for (int k = 0; k < n && k < 5; ++k) out[k] = c->prof[k];
    return BIB_OK;
}

bib_status bib_lattice_add_domain(bib_ctx* c, int64_t nx, int64_t ny, int64_t nz, const bib_lattice_params* p,
                                  int32_t* handle) {
    if (!c || !p || !handle) return fail(c, BIB_EINVAL, "null argument");
    if (nx < 3 || ny < 3 || nz < 3 || nx > 65535 || ny > 65535 || nz > 65535)
        return fail(c, BIB_EINVAL, "lattice dimensions must be in [3, 65535]");
    if (p->storage < BIB_STORAGE_F64 || p->storage > BIB_STORAGE_F16) return fail(c, BIB_EINVAL, "bad storage");
    if (p->collision < 0 || p->collision > BIB_COLLISION_TRT) return fail(c, BIB_EINVAL, "bad collision");
    if (!(p->omega > 0 && p->omega < 2)) return fail(c, BIB_EINVAL, "omega must lie in (0, 2)");
    if (p->use_phase && !(p->omega_inner > 0 && p->omega_inner < 2)) return fail(c, BIB_EINVAL, "omega_inner must lie in (0, 2)");
    if (p->periodic[0] == 0) return fail(c, BIB_EUNSUPPORTED, "the x axis must be periodic");
    if (!p->periodic[1] && p->wall_y == BIB_WALL_NONE) return fail(c, BIB_EINVAL, "non-periodic y needs a wall type");
    if (!p->periodic[2] && p->wall_z == BIB_WALL_NONE) return fail(c, BIB_EINVAL, "non-periodic z needs a wall type");
    if (!p->periodic[2] && p->wall_z == BIB_WALL_FD_VELOCITY)
        return fail(c, BIB_EUNSUPPORTED, "finite-difference velocity walls are implemented on y planes");
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(p->body_force[a])) return fail(c, BIB_EINVAL, "body force must be finite");
    for (int f = 0; f < 4; ++f)
        for (int a = 0; a < 3; ++a)
            if (!std::isfinite(p->wall_u[f][a])) return fail(c, BIB_EINVAL, "wall velocities must be finite");
    if (!(std::isfinite(p->trt_magic) && p->trt_magic >= 0)) return fail(c, BIB_EINVAL, "TRT magic parameter must be >= 0");
    if (!(std::isfinite(p->f16_scale) && p->f16_scale >= 0 && p->f16_scale <= 65504.0))
        return fail(c, BIB_EINVAL, "FP16 scale must lie in [0, 65504]");
    if (!p->periodic[1] && !p->periodic[2] && p->wall_y == BIB_WALL_FD_VELOCITY)
        return fail(c, BIB_EUNSUPPORTED, "finite-difference y walls need a periodic z axis");
    auto L = std::make_unique<Lattice>();
    LatticeDesc& d = L->d;
    d.nx = (int)nx;
    d.ny = (int)ny;
    d.nz = (int)nz;
    d.n = nx * ny * nz;
    // population / field arrays: 128-cell aligned, and offset by 384 cells so that the 19 + 12
    // concurrently streamed arrays do not start at a power-of-two distance from each other
    // (identical DRAM channel / bank interleaving for every stream)
    d.stride = (d.n + 127) / 128 * 128 + 384;
    d.px = p->periodic[0] != 0;
    d.py = p->periodic[1] != 0;
    d.pz = p->periodic[2] != 0;
    d.wall_y = d.py ? BIB_WALL_NONE : p->wall_y;
    d.wall_z = d.pz ? BIB_WALL_NONE : p->wall_z;
    d.collision = p->collision;
    d.use_phase = p->use_phase != 0;
    d.omega = p->omega;
    d.omega_inner = p->use_phase ? p->omega_inner : p->omega;
    d.trt_magic = p->trt_magic > 0 ? p->trt_magic : 0.25;
    // computeOmega, src/fsi/VariableViscosityDynamics.hh:131-141, for phase 0 and 1
    d.inv_n[0] = 1. / (double)d.nx;
    d.inv_n[1] = 1. / (double)d.ny;
    d.inv_n[2] = 1. / (double)d.nz;
    d.omega_c0 = d.omega * d.omega_inner / (0.0 * d.omega + (1. - 0.0) * d.omega_inner);
    d.omega_c1 = d.omega * d.omega_inner / (1.0 * d.omega + (1. - 1.0) * d.omega_inner);
    std::memcpy(d.wall_u, p->wall_u, sizeof(d.wall_u));
    std::memcpy(d.body, p->body_force, sizeof(d.body));
    const double sc = p->f16_scale > 0 ? p->f16_scale : 8192.0;
    d.scale = p->storage == BIB_STORAGE_F16 ? (float)sc : 1.0f;
    d.inv_scale = 1.0f / d.scale;
    L->storage = p->storage;
    d.fd_walls = (!d.py && d.wall_y == BIB_WALL_FD_VELOCITY) ? 1 : 0;
    const size_t pb = pop_bytes(p->storage) * Q * d.stride;
    const size_t fb = force_bytes(p->storage) * 3 * d.stride;
    const size_t wb = d.fd_walls ? pop_bytes(p->storage) * Q * 2 * (size_t)d.nx * d.nz : 0;
    const size_t ub = velocity_bytes(p->storage) * 4 * (size_t)d.n;  // (ux, uy, uz, 0) per cell
    void** bufs[6] = {&L->f[0], &L->f[1], &L->F[0], &L->F[1], &L->u, &L->wall};
    const size_t sizes[6] = {pb, pb, fb, fb, ub, wb};
    for (int k = 0; k < 6; ++k) {
        if (!sizes[k]) continue;
        cudaError_t e = dev_malloc(c, bufs[k], sizes[k]);
        if (e != cudaSuccess) {
            cudaGetLastError();
            for (int j = 0; j < k; ++j) cudaFree(*bufs[j]);
            return fail(c, BIB_ENOMEM, "device allocation of %zu bytes for a lattice buffer failed: %s", sizes[k],
                        cudaGetErrorString(e));
        }
        cudaMemsetAsync(*bufs[k], 0, sizes[k], c->stream);
    }
    if (d.use_phase) {
        if (dev_malloc(c, (void**)&L->phase, d.stride) != cudaSuccess) {
            cudaGetLastError();
            for (int j = 0; j < 6; ++j) cudaFree(*bufs[j]);
            return fail(c, BIB_ENOMEM, "device allocation of %zu bytes for the phase field failed", (size_t)d.stride);
        }
        cudaMemsetAsync(L->phase, 0, d.stride, c->stream);
    }
    L->target_clean = false;
    // external scalars start at zero, as Palabos cells do; every coupled step then
    // resets them to the body force before spreading (setExternalVector)
    BIB_CHECK_LAUNCH(c);
    *handle = (int32_t)c->lattices.size();
    L->handle = *handle;
    L->wait_err = c->d_flag + 1;
    L->vox_err = c->d_flag + 2;
    c->lattices.push_back(std::move(L));
    return BIB_OK;
}

bib_status bib_lattice_cells(bib_ctx* c, int32_t h, int64_t* n) {
    Lattice* L = get_lattice(c, h);
    if (!L || !n) return fail(c, BIB_EINVAL, "invalid lattice handle");
    *n = L->d.n;
    return BIB_OK;
}

bib_status bib_lattice_send(bib_ctx* c, int32_t h, const void* buf, size_t bytes, int32_t layout) {
    Lattice* L = get_lattice(c, h);
    if (!L || !buf) return fail(c, BIB_EINVAL, "invalid lattice handle or buffer");
    const int64_t n = L->d.n;
    Wire w{0};
    if (layout == BIB_LAYOUT_PALABOS_F64) w.per = Q + 4;
    else if (layout == BIB_LAYOUT_COPROCESSOR_F64) w.per = Q;
    else if (layout != BIB_LAYOUT_SOA_F64) return fail(c, BIB_EINVAL, "unknown layout %d", layout);
    const size_t want = (size_t)(w.per ? w.per : Q) * n * sizeof(double);
    if (bytes != want) return fail(c, BIB_EINVAL, "expected %zu bytes", want);
    bib_status st = import_populations(c, *L, static_cast<const double*>(buf), w);
    if (st) return st;
    if (w.per == Q + 4) {  // the force of the cells became the current external force
        L->target_clean = false;
        forces_touched(*L);
    }
    return BIB_OK;
}

bib_status bib_lattice_receive(bib_ctx* c, int32_t h, void* buf, size_t bytes, int32_t layout) {
    Lattice* L = get_lattice(c, h);
    if (!L || !buf) return fail(c, BIB_EINVAL, "invalid lattice handle or buffer");
    const int64_t n = L->d.n;
    const int per = layout == BIB_LAYOUT_PALABOS_F64 ? 23 : Q;
    const size_t want = (size_t)per * n * sizeof(double);
    if (layout != BIB_LAYOUT_SOA_F64 && layout != BIB_LAYOUT_PALABOS_F64 && layout != BIB_LAYOUT_COPROCESSOR_F64)
        return fail(c, BIB_EINVAL, "unknown layout");
    if (bytes != want) return fail(c, BIB_EINVAL, "expected %zu bytes", want);
    return export_populations(c, *L, static_cast<double*>(buf), Wire{layout == BIB_LAYOUT_SOA_F64 ? 0 : per});
}

bib_status bib_lattice_collide_and_stream(bib_ctx* c, int32_t h, int64_t nsteps) {
    return run_steps(c, h, nsteps, false, true);
}

bib_status bib_lattice_init_equilibrium(bib_ctx* c, int32_t h, const double* rho, const double* u) {
    Lattice* L = get_lattice(c, h);
    if (!L || !u) return fail(c, BIB_EINVAL, "invalid lattice handle or velocity");
    const int64_t n = L->d.n;
    // page-locked host arrays are read by the kernel directly; others are copied in first
    const double* mu = static_cast<const double*>(device_view_of_host(u, 3 * n * sizeof(double)));
    const double* mr = rho ? static_cast<const double*>(device_view_of_host(rho, n * sizeof(double))) : nullptr;
    if (mu && (!rho || mr)) {
        launch_init_equilibrium(*L, mr, mu, c->stream);
        launch_fd_walls(*L, L->cur, L->fe, c->stream);
        BIB_CHECK_LAUNCH(c);
        BIB_CUDA(c, cudaStreamSynchronize(c->stream));
        return BIB_OK;
    }
    double *dr = nullptr, *du = nullptr;
    bib_status st = device_buffer(c, &du, u, 3 * n);
    if (st) return st;
    if (rho) {
        st = device_buffer(c, &dr, rho, n);
        if (st) return st;
    }
    launch_init_equilibrium(*L, dr, du, c->stream);
    launch_fd_walls(*L, L->cur, L->fe, c->stream);
    BIB_CHECK_LAUNCH(c);
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(du);
    cudaFree(dr);
    return BIB_OK;
}

bib_status bib_lattice_set_force(bib_ctx* c, int32_t h, const double* F) {
    Lattice* L = get_lattice(c, h);
    if (!L || !F) return fail(c, BIB_EINVAL, "invalid lattice handle or force");
    double* d = nullptr;
    bib_status st = device_buffer(c, &d, F, 3 * L->d.n);
    if (st) return st;
    launch_force_import(*L, L->fe, d, c->stream);
    L->target_clean = false;
    forces_touched(*L);
    BIB_CHECK_LAUNCH(c);
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(d);
    return BIB_OK;
}

bib_status bib_lattice_get_force(bib_ctx* c, int32_t h, double* F) {
    Lattice* L = get_lattice(c, h);
    if (!L || !F) return fail(c, BIB_EINVAL, "invalid lattice handle or force");
    double* d = nullptr;
    bib_status st = device_buffer(c, &d, nullptr, 3 * L->d.n);
    if (st) return st;
    launch_force_export(*L, L->fe, d, c->stream);
    BIB_CHECK_LAUNCH(c);
    BIB_CUDA(c, cudaMemcpyAsync(F, d, 3 * L->d.n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(d);
    return BIB_OK;
}

bib_status bib_lattice_get_phase(bib_ctx* c, int32_t h, double* phase) {
    Lattice* L = get_lattice(c, h);
    if (!L || !phase) return fail(c, BIB_EINVAL, "invalid lattice handle or phase");
    if (!L->phase) return fail(c, BIB_ESTATE, "lattice was created with use_phase = 0");
    std::vector<uint8_t> h8((size_t)L->d.n);
    BIB_CUDA(c, cudaMemcpyAsync(h8.data(), L->phase, h8.size(), cudaMemcpyDeviceToHost, c->stream));
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    for (size_t k = 0; k < h8.size(); ++k) phase[k] = h8[k] ? 1.0 : 0.0;
    return BIB_OK;
}

bib_status bib_lattice_set_phase(bib_ctx* c, int32_t h, const double* phase) {
    Lattice* L = get_lattice(c, h);
    if (!L || !phase) return fail(c, BIB_EINVAL, "invalid lattice handle or phase");
    if (!L->phase) return fail(c, BIB_ESTATE, "lattice was created with use_phase = 0");
    double* d = nullptr;
    bib_status st = device_buffer(c, &d, phase, L->d.n);
    if (st) return st;
    launch_phase_import(*L, d, c->stream);
    BIB_CHECK_LAUNCH(c);
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(d);
    return BIB_OK;
}

bib_status bib_lattice_get_velocity(bib_ctx* c, int32_t h, double* u) {
    Lattice* L = get_lattice(c, h);
    if (!L || !u) return fail(c, BIB_EINVAL, "invalid lattice handle or velocity");
    if (double* m = static_cast<double*>(const_cast<void*>(device_view_of_host(u, 3 * L->d.n * sizeof(double))))) {
        launch_velocity_export(*L, m, c->stream);  // page-locked: written by the kernel directly
        BIB_CHECK_LAUNCH(c);
        BIB_CUDA(c, cudaStreamSynchronize(c->stream));
        return BIB_OK;
    }
    double* d = nullptr;
    bib_status st = device_buffer(c, &d, nullptr, 3 * L->d.n);
    if (st) return st;
    launch_velocity_export(*L, d, c->stream);
    BIB_CHECK_LAUNCH(c);
    BIB_CUDA(c, cudaMemcpyAsync(u, d, 3 * L->d.n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(d);
    return BIB_OK;
}

bib_status bib_shape_store(bib_ctx* c, const double* xyz, const int64_t* tri, int64_t nv, int64_t nt, int32_t* shape) {
    if (!c || !xyz || !tri || !shape) return fail(c, BIB_EINVAL, "null argument");
    if (nv < 4 || nt < 4 || nv > (1 << 24) || nt > (1 << 25)) return fail(c, BIB_EINVAL, "bad mesh size");
    auto S = std::make_unique<ShapeHost>();
    std::string why;
    if (!build_shape(*S, xyz, tri, nv, nt, why)) return fail(c, BIB_EINVAL, "invalid mesh: %s", why.c_str());
    bib_status st;
    if ((st = upload(c, &S->dev.rest, S->rest)) || (st = upload(c, &S->dev.tri, S->tri)) ||
        (st = upload(c, &S->dev.tri_area, S->tri_area)) || (st = upload(c, &S->dev.links, S->links)) ||
        (st = upload(c, &S->dev.link_len, S->link_len)) || (st = upload(c, &S->dev.pairs, S->pairs)) ||
        (st = upload(c, &S->dev.pair_cs, S->pair_cs)) || (st = upload(c, &S->dev.inc_off, S->inc_off)) ||
        (st = upload(c, &S->dev.inc, S->inc)) || (st = upload(c, &S->dev.tri_rest_f, S->tri_rest_f)) ||
        (st = upload(c, &S->dev.tri_area_f, S->tri_area_f)) || (st = upload(c, &S->dev.pair_cs_f, S->pair_cs_f)) ||
        (st = upload(c, &S->dev.tri4, S->tri4)))
        return st;
    S->dev.nv = (int)nv;
    S->dev.nt = (int)nt;
    S->dev.nl = (int)S->link_len.size();
    S->dev.np = (int)S->pair_cs.size() / 2;
    S->dev.area = S->area;
    S->dev.volume = S->volume;
    *shape = (int32_t)c->shapes.size();
    c->shapes.push_back(std::move(S));
    return BIB_OK;
}

bib_status bib_shape_info(bib_ctx* c, int32_t shape, double* out) {
    if (!c || !out || shape < 0 || shape >= (int32_t)c->shapes.size()) return fail(c, BIB_EINVAL, "invalid shape");
    const ShapeHost& S = *c->shapes[shape];
    out[0] = S.area;
    out[1] = S.volume;
    out[2] = (double)S.link_len.size();
    out[3] = (double)(S.pair_cs.size() / 2);
    out[4] = (double)(S.rest.size() / 3);
    out[5] = (double)S.tri_area.size();
    return BIB_OK;
}

bib_status bib_ib_configure(bib_ctx* c, int32_t h, const bib_ib_params* p) {
    Lattice* L = get_lattice(c, h);
    if (!L || !p) return fail(c, BIB_EINVAL, "invalid lattice handle or parameters");
    if (p->dirac != BIB_DIRAC_ROMA && p->dirac != BIB_DIRAC_PESKIN) return fail(c, BIB_EINVAL, "bad dirac");
    if (p->spread_mode != BIB_SPREAD_ATOMIC && p->spread_mode != BIB_SPREAD_DETERMINISTIC)
        return fail(c, BIB_EINVAL, "bad spread mode");
    if (L->d.n >= (int64_t)0xffffffff) return fail(c, BIB_EUNSUPPORTED, "lattice too large for 32-bit cell keys");
    if (p->field_offset != std::floor(p->field_offset)) return fail(c, BIB_EINVAL, "field offset must be integral");
    if (L->ib.has_pipe && p->spread_mode == BIB_SPREAD_DETERMINISTIC)
        return fail(c, BIB_EUNSUPPORTED, "deterministic spreading does not blend kernels near a pipe boundary");
    L->ib.dirac = p->dirac;
    L->ib.spread_mode = p->spread_mode;
    L->ib.offset = p->field_offset;
    // the spreading buffers depend on the mode: re-upload the particles on the next step
    bib_status pst = pull_particles(c, *L);
    if (pst) return pst;
    if (!L->parts.empty()) L->particles_dirty = true;
    drop_graphs(c, h);
    return BIB_OK;
}

// Interaction changes alter kernel arguments captured in graphs and batch tables
static void interactions_changed(bib_ctx* c, int32_t h) {
    drop_graphs(c, h);
    for (auto& B : c->batches)
        if (B) B->free_tables();
}

bib_status bib_ib_set_pipe_boundary(bib_ctx* c, int32_t h, double y0, double z0, double radius) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    if (!std::isfinite(y0) || !std::isfinite(z0) || !std::isfinite(radius)) return fail(c, BIB_EINVAL, "bad pipe geometry");
    if (radius > 0 && L->ib.spread_mode == BIB_SPREAD_DETERMINISTIC)
        return fail(c, BIB_EUNSUPPORTED, "deterministic spreading does not blend kernels near a pipe boundary");
    L->ib.has_pipe = radius > 0;
    L->ib.pipe_y0 = y0;
    L->ib.pipe_z0 = z0;
    L->ib.pipe_r = radius > 0 ? radius : 0.0;
    interactions_changed(c, h);  // the IB description is captured by graphs and batch tables
    return BIB_OK;
}

static bib_status check_potential(bib_ctx* c, const bib_potential* p) {
    if (!p) return fail(c, BIB_EINVAL, "null potential");
    if (p->kind != BIB_POTENTIAL_MORSE && p->kind != BIB_POTENTIAL_SPRING) return fail(c, BIB_EINVAL, "bad potential kind");
    if (!(p->r0 > 0 && std::isfinite(p->r0)) || !std::isfinite(p->strength) || !std::isfinite(p->beta))
        return fail(c, BIB_EINVAL, "potential parameters must be finite, with a positive cutoff");
    return BIB_OK;
}


bib_status bib_add_wall_interaction(bib_ctx* c, int32_t h, int32_t axis, double lo, double hi, const bib_potential* p) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    bib_status st = check_potential(c, p);
    if (st) return st;
    if (axis < 0 || axis > 2 || !(lo < hi)) return fail(c, BIB_EINVAL, "wall interaction needs axis 0..2 and lo < hi");
    if (L->inter.nwall >= BIB_MAX_WALL_INTERACTIONS) return fail(c, BIB_EINVAL, "too many wall interactions");
    const int w = L->inter.nwall++;
    L->inter.wall_axis[w] = axis;
    L->inter.wall_lo[w] = lo;
    L->inter.wall_hi[w] = hi;
    L->inter.wall[w] = PotentialDev{p->kind, p->r0, p->beta, p->strength};
    interactions_changed(c, h);
    return BIB_OK;
}

bib_status bib_add_pipe_wall_interaction(bib_ctx* c, int32_t h, double y0, double z0, double radius,
                                         const bib_potential* p) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    bib_status st = check_potential(c, p);
    if (st) return st;
    if (!(radius > 0) || !std::isfinite(y0) || !std::isfinite(z0)) return fail(c, BIB_EINVAL, "bad pipe");
    if (L->inter.nwall >= BIB_MAX_WALL_INTERACTIONS) return fail(c, BIB_EINVAL, "too many wall interactions");
    const int w = L->inter.nwall++;
    L->inter.wall_axis[w] = 3;
    L->inter.wall_lo[w] = y0;
    L->inter.wall_hi[w] = z0;
    L->inter.wall_r[w] = radius;
    L->inter.wall[w] = PotentialDev{p->kind, p->r0, p->beta, p->strength};
    interactions_changed(c, h);
    return BIB_OK;
}

bib_status bib_add_pp_interaction(bib_ctx* c, int32_t h, const bib_potential* p) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    bib_status st = check_potential(c, p);
    if (st) return st;
    if (L->inter.npp >= BIB_MAX_PP_INTERACTIONS) return fail(c, BIB_EINVAL, "too many particle-particle interactions");
    if (p->search != BIB_PAIR_SEARCH_ALL && p->search != BIB_PAIR_SEARCH_GRID) return fail(c, BIB_EINVAL, "bad pair search");
    if (L->inter.npp > 0 && p->search != L->inter.pp_search)
        return fail(c, BIB_EINVAL, "the particle-particle interactions of a lattice use one pair search");
    // the reference limits the cutoff to the delta kernel's half support - 1/2
    // (ImmersedBoundaryDynamics_forces.hh:346-349)
    const double limit = (L->ib.dirac == BIB_DIRAC_PESKIN ? 2.0 : 1.5) - 0.5;
    if (p->r0 > limit) return fail(c, BIB_EINVAL, "interaction cutoff %g exceeds %g", p->r0, limit);
    L->inter.pp[L->inter.npp++] = PotentialDev{p->kind, p->r0, p->beta, p->strength};
    L->inter.pp_search = p->search;
    L->inter.pp_cut = std::max(L->inter.pp_cut, p->r0);
    // the pair search buffers are sized with the particles: re-upload them on the next step
    st = pull_particles(c, *L);
    if (st) return st;
    if (!L->parts.empty()) L->particles_dirty = true;
    interactions_changed(c, h);
    return BIB_OK;
}

bib_status bib_clear_interactions(bib_ctx* c, int32_t h) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    L->inter = Interactions{};
    interactions_changed(c, h);
    return BIB_OK;
}

bib_status bib_particle_add(bib_ctx* c, int32_t h, int32_t shape, int32_t model, const double* params,
                            const double* xyz, int32_t* pid) {
    Lattice* L = get_lattice(c, h);
    if (!L || !params || !pid) return fail(c, BIB_EINVAL, "invalid lattice handle or argument");
    if (shape < 0 || shape >= (int32_t)c->shapes.size()) return fail(c, BIB_EINVAL, "invalid shape %d", shape);
    if (model < BIB_MODEL_CAPSULE_NEOHOOKEAN || model > BIB_MODEL_SKALAK_BENDING) return fail(c, BIB_EINVAL, "bad model");
    const ShapeHost& S = *c->shapes[shape];
    const int nv = (int)(S.rest.size() / 3);
    if (model == BIB_MODEL_RBC_WLCPOW || model == BIB_MODEL_SKALAK_BENDING) {
        if (!(params[BIB_P_VOL_DESIRED] != 0)) return fail(c, BIB_EINVAL, "vol_desired must be non-zero");
    }
    for (int k = 0; k < BIB_P_COUNT; ++k)
        if (!std::isfinite(params[k])) return fail(c, BIB_EINVAL, "membrane parameter %d is not finite", k);
    if (xyz)
        for (int k = 0; k < 3 * nv; ++k)
            if (!std::isfinite(xyz[k])) return fail(c, BIB_EINVAL, "vertex coordinate %d is not finite", k);
    bib_status pst = pull_particles(c, *L);
    if (pst) return pst;
    ParticleHost ph;
    ph.shape = shape;
    ph.model = model;
    ph.v0 = (int)(L->host_pos.size() / 3);
    ph.nv = nv;
    ph.prm.assign(params, params + BIB_P_COUNT);
    std::vector<double> pos(xyz ? xyz : S.rest.data(), (xyz ? xyz : S.rest.data()) + 3 * nv);
    double st[STATS];
    particle_update(S, pos.data(), st);
    remap_com(L->d, pos.data(), nv, st);
    L->host_pos.insert(L->host_pos.end(), pos.begin(), pos.end());
    L->host_stats.insert(L->host_stats.end(), st, st + STATS);
    L->parts.push_back(ph);
    L->particles_dirty = true;
    *pid = (int32_t)L->parts.size() - 1;
    return BIB_OK;
}

bib_status bib_particle_count(bib_ctx* c, int32_t h, int32_t* n) {
    Lattice* L = get_lattice(c, h);
    if (!L || !n) return fail(c, BIB_EINVAL, "invalid lattice handle");
    *n = (int32_t)L->parts.size();
    return BIB_OK;
}

bib_status bib_particle_info(bib_ctx* c, int32_t h, int32_t pid, int32_t* out) {
    Lattice* L = get_lattice(c, h);
    if (!L || !out || pid < 0 || pid >= (int32_t)L->parts.size()) return fail(c, BIB_EINVAL, "invalid particle");
    out[0] = L->parts[pid].shape;
    out[1] = L->parts[pid].model;
    out[2] = L->parts[pid].nv;
    return BIB_OK;
}

bib_status bib_total_vertices(bib_ctx* c, int32_t h, int64_t* n) {
    Lattice* L = get_lattice(c, h);
    if (!L || !n) return fail(c, BIB_EINVAL, "invalid lattice handle");
    int64_t s = 0;
    for (auto& p : L->parts) s += p.nv;
    *n = s;
    return BIB_OK;
}

bib_status bib_particle_get(bib_ctx* c, int32_t h, int32_t pid, double* pos, double* vel, double* force) {
    Lattice* L = get_lattice(c, h);
    if (!L || pid < 0 || pid >= (int32_t)L->parts.size()) return fail(c, BIB_EINVAL, "invalid particle");
    const ParticleHost& ph = L->parts[pid];
    const size_t off = 3 * (size_t)ph.v0, cnt = 3 * (size_t)ph.nv;
    if (L->particles_dirty) {
        if (pos) std::memcpy(pos, L->host_pos.data() + off, cnt * 8);
        if (vel) std::memset(vel, 0, cnt * 8);
        if (force) std::memset(force, 0, cnt * 8);
        return BIB_OK;
    }
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    if (pos) BIB_CUDA(c, cudaMemcpy(pos, L->pos[L->pcur] + off, cnt * 8, cudaMemcpyDeviceToHost));
    if (vel) BIB_CUDA(c, cudaMemcpy(vel, L->vel + off, cnt * 8, cudaMemcpyDeviceToHost));
    if (force) BIB_CUDA(c, cudaMemcpy(force, L->force + off, cnt * 8, cudaMemcpyDeviceToHost));
    return BIB_OK;
}

bib_status bib_particle_set_positions(bib_ctx* c, int32_t h, int32_t pid, const double* pos) {
    Lattice* L = get_lattice(c, h);
    if (!L || !pos || pid < 0 || pid >= (int32_t)L->parts.size()) return fail(c, BIB_EINVAL, "invalid particle");
    const ParticleHost& ph = L->parts[pid];
    bib_status pst = pull_particles(c, *L);
    if (pst) return pst;
    std::memcpy(L->host_pos.data() + 3 * (size_t)ph.v0, pos, 3 * (size_t)ph.nv * 8);
    particle_update(*c->shapes[ph.shape], L->host_pos.data() + 3 * (size_t)ph.v0, L->host_stats.data() + STATS * pid);
    L->particles_dirty = true;
    return BIB_OK;
}

bib_status bib_particles_download(bib_ctx* c, int32_t h, double* pos, double* stats) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    if (L->particles_dirty) {
        if (pos) std::memcpy(pos, L->host_pos.data(), L->host_pos.size() * 8);
        if (stats) std::memcpy(stats, L->host_stats.data(), L->host_stats.size() * 8);
        return BIB_OK;
    }
    if (pos && L->nvert) BIB_CUDA(c, cudaMemcpyAsync(pos, L->pos[L->pcur], 3 * (size_t)L->nvert * 8, cudaMemcpyDeviceToHost, c->stream));
    if (stats && !L->parts.empty())
        BIB_CUDA(c, cudaMemcpyAsync(stats, L->stats, STATS * L->parts.size() * 8, cudaMemcpyDeviceToHost, c->stream));
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    return BIB_OK;
}

bib_status bib_particles_upload(bib_ctx* c, int32_t h, const double* pos) {
    Lattice* L = get_lattice(c, h);
    if (!L || !pos) return fail(c, BIB_EINVAL, "invalid lattice handle or positions");
    if (L->particles_dirty) {  // not uploaded yet: replace the host copies
        std::memcpy(L->host_pos.data(), pos, L->host_pos.size() * 8);
        for (size_t p = 0; p < L->parts.size(); ++p) {
            const ParticleHost& ph = L->parts[p];
            particle_update(*c->shapes[ph.shape], L->host_pos.data() + 3 * (size_t)ph.v0, L->host_stats.data() + STATS * p);
        }
        return BIB_OK;
    }
    if (L->nvert == 0) return BIB_OK;
    // into the move target, then the end of a step: area / volume / centre (and the periodic
    // remap of the centre) of the new positions, the parity flip, the voxelization
    BIB_CUDA(c, cudaMemcpyAsync(L->pos[1 - L->pcur], pos, 3 * (size_t)L->nvert * 8, cudaMemcpyHostToDevice, c->stream));
    launch_particle_update(*L, c->stream);
    L->pcur = 1 - L->pcur;
    if (L->phase) launch_voxelize(*L, L->pos[L->pcur], c->stream);
    BIB_CHECK_LAUNCH(c);
    return BIB_OK;
}

bib_status bib_particles_download_async(bib_ctx* c, int32_t h, double* pos, double* stats, int32_t slot) {
    Lattice* L = get_lattice(c, h);
    if (!L || slot < 0 || slot >= 8) return fail(c, BIB_EINVAL, "invalid lattice handle or slot");
    if (L->particles_dirty) {  // not uploaded yet: the host copies are the state
        if (pos) std::memcpy(pos, L->host_pos.data(), L->host_pos.size() * 8);
        if (stats) std::memcpy(stats, L->host_stats.data(), L->host_stats.size() * 8);
    } else {
        if (pos && L->nvert)
            BIB_CUDA(c, cudaMemcpyAsync(pos, L->pos[L->pcur], 3 * (size_t)L->nvert * 8, cudaMemcpyDeviceToHost, c->stream));
        if (stats && !L->parts.empty()) {
            // a page-locked buffer is written by a small kernel over the link: no copy-engine
            // hand-over between the step graphs of a step-then-read loop
            const size_t n = STATS * L->parts.size();
            if (double* m = static_cast<double*>(const_cast<void*>(device_view_of_host(stats, n * 8)))) {
                launch_copy_f64(m, L->stats, n, c->stream);
                BIB_CHECK_LAUNCH(c);
            } else {
                BIB_CUDA(c, cudaMemcpyAsync(stats, L->stats, n * 8, cudaMemcpyDeviceToHost, c->stream));
            }
        }
    }
    BIB_CUDA(c, cudaEventRecord(c->dl_ev[slot], c->stream));
    return BIB_OK;
}

bib_status bib_download_wait(bib_ctx* c, int32_t slot) {
    if (!c || slot < 0 || slot >= 8) return fail(c, BIB_EINVAL, "invalid slot");
    BIB_CUDA(c, cudaEventSynchronize(c->dl_ev[slot]));
    return BIB_OK;
}

bib_status bib_particle_stats(bib_ctx* c, int32_t h, int32_t pid, double* out) {
    Lattice* L = get_lattice(c, h);
    if (!L || !out || pid < 0 || pid >= (int32_t)L->parts.size()) return fail(c, BIB_EINVAL, "invalid particle");
    const ParticleHost& ph = L->parts[pid];
    std::vector<double> pos(3 * (size_t)ph.nv);
    bib_status st = bib_particle_get(c, h, pid, pos.data(), nullptr, nullptr);
    if (st) return st;
    double s[STATS];
    if (L->particles_dirty) {
        std::memcpy(s, L->host_stats.data() + STATS * pid, sizeof(s));
    } else {
        BIB_CUDA(c, cudaMemcpy(s, L->stats + STATS * pid, sizeof(s), cudaMemcpyDeviceToHost));
    }
    std::memcpy(out, s, sizeof(s));
    moment_of_inertia(*c->shapes[ph.shape], pos.data(), out + STATS);
    return BIB_OK;
}

bib_status bib_total_volume(bib_ctx* c, int32_t h, double* v) {
    Lattice* L = get_lattice(c, h);
    if (!L || !v) return fail(c, BIB_EINVAL, "invalid lattice handle");
    std::vector<double> st(STATS * L->parts.size());
    bib_status s = bib_particles_download(c, h, nullptr, st.data());
    if (s) return s;
    double tot = 0;
    for (size_t p = 0; p < L->parts.size(); ++p) tot += st[STATS * p + 1];
    *v = tot;
    return BIB_OK;
}

bib_status bib_ibm_step(bib_ctx* c, int32_t h) { return run_steps(c, h, 1, true, false); }

bib_status bib_step(bib_ctx* c, int32_t h, int64_t nsteps) { return run_steps(c, h, nsteps, true, true); }

bib_status bib_step_timed(bib_ctx* c, int32_t h, int64_t nsteps, double* ms) {
    if (!c || !ms) return fail(c, BIB_EINVAL, "null argument");
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle %d", h);
    bib_status st = sync_particles(c, *L);  // uploads happen outside the timed region
    if (st) return st;
    cudaEvent_t a, b;
    BIB_CUDA(c, cudaEventCreate(&a));
    BIB_CUDA(c, cudaEventCreate(&b));
    BIB_CUDA(c, cudaEventRecord(a, c->stream));
    st = run_steps(c, h, nsteps, true, true);
    BIB_CUDA(c, cudaEventRecord(b, c->stream));
    BIB_CUDA(c, cudaEventSynchronize(b));
    float f = 0;
    BIB_CUDA(c, cudaEventElapsedTime(&f, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = f;
    return st;
}

bib_status bib_coprocessor_domain_params(double omega, int32_t storage, int32_t collision, bib_lattice_params* p) {
    if (!p || !(omega > 0.0 && omega < 2.0)) return BIB_EINVAL;
    if (storage != BIB_STORAGE_F64 && storage != BIB_STORAGE_F32 && storage != BIB_STORAGE_F16) return BIB_EINVAL;
    if (collision != BIB_COLLISION_BGK && collision != BIB_COLLISION_BGK_GUO_VOF) return BIB_EINVAL;
    std::memset(p, 0, sizeof(*p));
    p->periodic[0] = p->periodic[1] = p->periodic[2] = 1;
    p->collision = collision;
    p->storage = storage;
    p->wall_y = p->wall_z = BIB_WALL_NONE;
    p->omega = p->omega_inner = omega;
    p->trt_magic = 0.25;
    return BIB_OK;
}

bib_status bib_step_kernel_count(bib_ctx* c, int32_t h, int32_t* kernels_per_step) {
    if (!c || !kernels_per_step) return fail(c, BIB_EINVAL, "null argument");
    if (!get_lattice(c, h)) return fail(c, BIB_EINVAL, "invalid lattice handle %d", h);
    // two-step graphs hold two steps; one-step graphs one
    int best = -1;
    for (const auto& kv : c->graphs)
        if (kv.first.first == h && kv.second.exec) {
            const int steps = kv.first.second >= 8 ? 2 : 1;
            best = std::max(best, (kv.second.kernels + steps - 1) / steps);
        }
    if (best < 0) return fail(c, BIB_EINVAL, "lattice %d has no captured step graph yet", h);
    *kernels_per_step = best;
    return BIB_OK;
}

bib_status bib_check_health(bib_ctx* c, int32_t h) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    BIB_CUDA(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
    launch_nan_scan(*L, c->d_flag, c->stream);
    BIB_CHECK_LAUNCH(c);
    int flag[3] = {0, 0, 0};
    BIB_CUDA(c, cudaMemcpyAsync(flag, c->d_flag, 3 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    if (flag[1]) {
        BIB_CUDA(c, cudaMemsetAsync(c->d_flag + 1, 0, sizeof(int), c->stream));
        return fail(c, BIB_ETIMEOUT, "a bounded device wait gave up; the results of that step are invalid");
    }
    if (flag[2]) {
        BIB_CUDA(c, cudaMemsetAsync(c->d_flag + 2, 0, sizeof(int), c->stream));
        return fail(c, BIB_EOVERFLOW, "voxelization: a lattice column was crossed by more than %d membrane triangles, or "
                    "a triangle was wider than the lattice; the phase field of that step is incomplete", kVoxelCap);
    }
    if (flag[0]) return fail(c, BIB_ENAN, "populations contain NaN or Inf");
    if (!L->particles_dirty && L->nvert) {
        std::vector<double> pos(3 * (size_t)L->nvert);
        BIB_CUDA(c, cudaMemcpy(pos.data(), L->pos[L->pcur], pos.size() * 8, cudaMemcpyDeviceToHost));
        for (double v : pos)
            if (!std::isfinite(v)) return fail(c, BIB_ENAN, "vertex positions contain NaN or Inf");
    }
    return BIB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- checkpoints
// One file per lattice: the reference's lattice checkpoint (parallelIO::save,
// io/multiBlockWriter3D.cpp:201), its particle checkpoint (save_checkpoint,
// ImmersedBoundaryDynamics_io.hh:17-72, one pack per particle) and its iteration counter
// (Time::write_checkpoint, Time.h:20-27) in one versioned binary.  The device buffers are
// written in their own storage type, so a run resumed from a checkpoint continues bit for
// bit (with deterministic spreading).  Layout, all little-endian:
//   CkptHeader | f[cur] (19 x stride) | wall buffer (FD walls) | F[0] | F[1] (3 x stride each)
//   | phase (stride bytes, use_phase) | cell types (n bytes, when set)
//   | per particle: CkptParticle + BIB_P_COUNT doubles | positions, velocities, forces (3 x nvert
//   each) | STATS doubles per particle | 64-bit checksum of everything before it.
namespace {

constexpr char kCkptMagic[8] = {'B', 'I', 'B', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t kCkptVersion = 1;

struct CkptHeader {
    char magic[8];
    uint32_t version, header_bytes;
    int32_t nx, ny, nz, storage, collision, use_phase, has_types, fd_walls;
    int32_t px, py, pz, wall_y, wall_z;
    int32_t cur, fe, target_clean, nparts, p_count;
    int64_t stride, nvert;
    uint64_t iteration;
    double omega, omega_inner, trt_magic, scale;
    double body[3], wall_u[4][3];
};

struct CkptParticle {
    int32_t shape, model, nv, nt;
};

// 64-bit multiply-xorshift hash over the byte stream, 8 bytes at a time
struct Checksum {
    uint64_t h = 0x9e3779b97f4a7c15ull;
    uint64_t carry = 0;
    int nc = 0;
    void word(uint64_t w) {
        h ^= w;
        h *= 0xbf58476d1ce4e5b9ull;
        h ^= h >> 31;
    }
    void add(const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        size_t i = 0;
        while (nc && i < n) {
            carry |= (uint64_t)b[i++] << (8 * nc);
            if (++nc == 8) word(carry), carry = 0, nc = 0;
        }
        for (; i + 8 <= n; i += 8) {
            uint64_t w;
            std::memcpy(&w, b + i, 8);
            word(w);
        }
        for (; i < n; ++i) {
            carry |= (uint64_t)b[i] << (8 * nc);
            ++nc;
        }
    }
    uint64_t value() const {
        Checksum t = *this;
        if (t.nc) t.word(t.carry ^ ((uint64_t)t.nc << 56));
        return t.h;
    }
};

struct CkptFile {
    FILE* f = nullptr;
    Checksum sum;
    ~CkptFile() {
        if (f) fclose(f);
    }
    bool put(const void* p, size_t n) {
        sum.add(p, n);
        return fwrite(p, 1, n, f) == n;
    }
    bool get(void* p, size_t n) {
        if (fread(p, 1, n, f) != n) return false;
        sum.add(p, n);
        return true;
    }
};

constexpr size_t kCkptChunk = (size_t)64 << 20;

bib_status ckpt_put_device(bib_ctx* c, CkptFile& F, const void* dev, size_t bytes, std::vector<unsigned char>& buf) {
    for (size_t o = 0; o < bytes; o += kCkptChunk) {
        const size_t n = std::min(kCkptChunk, bytes - o);
        buf.resize(n);
        BIB_CUDA(c, cudaMemcpy(buf.data(), static_cast<const unsigned char*>(dev) + o, n, cudaMemcpyDeviceToHost));
        if (!F.put(buf.data(), n)) return fail(c, BIB_EINVAL, "checkpoint write failed");
    }
    return BIB_OK;
}

bib_status ckpt_get_device(bib_ctx* c, CkptFile& F, void* dev, size_t bytes, std::vector<unsigned char>& buf) {
    for (size_t o = 0; o < bytes; o += kCkptChunk) {
        const size_t n = std::min(kCkptChunk, bytes - o);
        buf.resize(n);
        if (!F.get(buf.data(), n)) return fail(c, BIB_EINVAL, "checkpoint file is truncated");
        BIB_CUDA(c, cudaMemcpy(static_cast<unsigned char*>(dev) + o, buf.data(), n, cudaMemcpyHostToDevice));
    }
    return BIB_OK;
}

size_t wall_bytes(const Lattice& L) {
    return L.d.fd_walls ? pop_bytes(L.storage) * Q * 2 * (size_t)L.d.nx * L.d.nz : 0;
}

CkptHeader ckpt_header(const Lattice& L) {
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kCkptMagic, 8);
    h.version = kCkptVersion;
    h.header_bytes = sizeof(CkptHeader);
    h.nx = L.d.nx, h.ny = L.d.ny, h.nz = L.d.nz;
    h.storage = L.storage, h.collision = L.d.collision, h.use_phase = L.d.use_phase;
    h.has_types = L.celltype != nullptr, h.fd_walls = L.d.fd_walls;
    h.px = L.d.px, h.py = L.d.py, h.pz = L.d.pz, h.wall_y = L.d.wall_y, h.wall_z = L.d.wall_z;
    h.cur = L.cur, h.fe = L.fe, h.target_clean = L.target_clean;
    h.nparts = (int32_t)L.parts.size(), h.p_count = BIB_P_COUNT;
    h.stride = L.d.stride;
    h.nvert = L.nvert;
    h.iteration = L.iteration;
    h.omega = L.d.omega, h.omega_inner = L.d.omega_inner, h.trt_magic = L.d.trt_magic, h.scale = L.d.scale;
    std::memcpy(h.body, L.d.body, sizeof(h.body));
    std::memcpy(h.wall_u, L.d.wall_u, sizeof(h.wall_u));
    return h;
}

}  // namespace

extern "C" {

bib_status bib_lattice_iteration(bib_ctx* c, int32_t h, int64_t* it) {
    Lattice* L = get_lattice(c, h);
    if (!L || !it) return fail(c, BIB_EINVAL, "invalid lattice handle or argument");
    *it = (int64_t)L->iteration;
    return BIB_OK;
}

bib_status bib_ibm_init(bib_ctx* c, int32_t h) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    bib_status st = sync_particles(c, *L);
    if (st) return st;
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    return BIB_OK;
}

bib_status bib_checkpoint_save(bib_ctx* c, int32_t h, const char* path) {
    Lattice* L = get_lattice(c, h);
    if (!L || !path) return fail(c, BIB_EINVAL, "invalid lattice handle or path");
    bib_status st = sync_particles(c, *L);
    if (st) return st;
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    CkptFile F;
    F.f = fopen(path, "wb");
    if (!F.f) return fail(c, BIB_EINVAL, "cannot open %s for writing", path);
    const CkptHeader hd = ckpt_header(*L);
    if (!F.put(&hd, sizeof(hd))) return fail(c, BIB_EINVAL, "checkpoint write failed");
    std::vector<unsigned char> buf;
    const size_t pb = pop_bytes(L->storage) * Q * (size_t)L->d.stride;
    const size_t fb = force_bytes(L->storage) * 3 * (size_t)L->d.stride;
    if ((st = ckpt_put_device(c, F, L->f[L->cur], pb, buf))) return st;
    if (L->d.fd_walls && (st = ckpt_put_device(c, F, L->wall, wall_bytes(*L), buf))) return st;
    for (int k = 0; k < 2; ++k)
        if ((st = ckpt_put_device(c, F, L->F[k], fb, buf))) return st;
    if (L->phase && (st = ckpt_put_device(c, F, L->phase, (size_t)L->d.stride, buf))) return st;
    if (L->celltype && (st = ckpt_put_device(c, F, L->celltype, (size_t)L->d.n, buf))) return st;
    for (const ParticleHost& ph : L->parts) {
        const ShapeHost& S = *c->shapes[ph.shape];
        const CkptParticle cp{ph.shape, ph.model, ph.nv, (int32_t)S.tri_area.size()};
        if (!F.put(&cp, sizeof(cp)) || !F.put(ph.prm.data(), BIB_P_COUNT * sizeof(double)))
            return fail(c, BIB_EINVAL, "checkpoint write failed");
    }
    if (L->nvert) {
        const size_t vb = 3 * (size_t)L->nvert * sizeof(double);
        if ((st = ckpt_put_device(c, F, L->pos[L->pcur], vb, buf))) return st;
        if ((st = ckpt_put_device(c, F, L->vel, vb, buf))) return st;
        if ((st = ckpt_put_device(c, F, L->force, vb, buf))) return st;
        if ((st = ckpt_put_device(c, F, L->stats, STATS * L->parts.size() * sizeof(double), buf))) return st;
    }
    const uint64_t sum = F.sum.value();
    if (fwrite(&sum, 1, sizeof(sum), F.f) != sizeof(sum) || fflush(F.f) != 0)
        return fail(c, BIB_EINVAL, "checkpoint write failed");
    return BIB_OK;
}

bib_status bib_checkpoint_load(bib_ctx* c, int32_t h, const char* path) {
    Lattice* L = get_lattice(c, h);
    if (!L || !path) return fail(c, BIB_EINVAL, "invalid lattice handle or path");
    CkptFile F;
    F.f = fopen(path, "rb");
    if (!F.f) return fail(c, BIB_EINVAL, "cannot open %s for reading", path);
    CkptHeader hd;
    if (!F.get(&hd, sizeof(hd))) return fail(c, BIB_EINVAL, "checkpoint file is truncated");
    if (std::memcmp(hd.magic, kCkptMagic, 8) != 0) return fail(c, BIB_EINVAL, "%s is not a biblbm_gb300 checkpoint", path);
    if (hd.version != kCkptVersion || hd.header_bytes != sizeof(CkptHeader) || hd.p_count != BIB_P_COUNT)
        return fail(c, BIB_EUNSUPPORTED, "checkpoint format version %u is not supported", hd.version);
    // the lattice must be configured as the one that was saved
    const CkptHeader me = ckpt_header(*L);
    const bool same = hd.nx == me.nx && hd.ny == me.ny && hd.nz == me.nz && hd.storage == me.storage &&
                      hd.collision == me.collision && hd.use_phase == me.use_phase && hd.fd_walls == me.fd_walls &&
                      hd.px == me.px && hd.py == me.py && hd.pz == me.pz && hd.wall_y == me.wall_y &&
                      hd.wall_z == me.wall_z && hd.stride == me.stride && hd.omega == me.omega &&
                      hd.omega_inner == me.omega_inner && hd.trt_magic == me.trt_magic && hd.scale == me.scale &&
                      std::memcmp(hd.body, me.body, sizeof(hd.body)) == 0 &&
                      std::memcmp(hd.wall_u, me.wall_u, sizeof(hd.wall_u)) == 0;
    if (!same) return fail(c, BIB_EINVAL, "checkpoint was written by a lattice of another configuration");
    if (hd.nparts < 0 || hd.nvert < 0 || hd.nvert > (int64_t)1 << 31 || hd.cur < 0 || hd.cur > 1 || hd.fe < 0 || hd.fe > 1)
        return fail(c, BIB_EINVAL, "corrupt checkpoint header");
    // read everything host-side first (particles) and validate it before touching the lattice
    std::vector<unsigned char> buf;
    const size_t pb = pop_bytes(L->storage) * Q * (size_t)L->d.stride;
    const size_t fb = force_bytes(L->storage) * 3 * (size_t)L->d.stride;
    const long body_at = ftell(F.f);
    size_t skip = pb + wall_bytes(*L) + 2 * fb + (hd.use_phase ? (size_t)hd.stride : 0) + (hd.has_types ? (size_t)L->d.n : 0);
    // pass 1: checksum of the whole file and the particle records
    {
        std::vector<unsigned char> tmp;
        for (size_t o = 0; o < skip; o += kCkptChunk) {
            const size_t n = std::min(kCkptChunk, skip - o);
            tmp.resize(n);
            if (!F.get(tmp.data(), n)) return fail(c, BIB_EINVAL, "checkpoint file is truncated");
        }
    }
    std::vector<ParticleHost> parts(hd.nparts);
    int64_t vtot = 0;
    for (int32_t p = 0; p < hd.nparts; ++p) {
        CkptParticle cp;
        ParticleHost& ph = parts[p];
        ph.prm.resize(BIB_P_COUNT);
        if (!F.get(&cp, sizeof(cp)) || !F.get(ph.prm.data(), BIB_P_COUNT * sizeof(double)))
            return fail(c, BIB_EINVAL, "checkpoint file is truncated");
        if (cp.shape < 0 || cp.shape >= (int32_t)c->shapes.size())
            return fail(c, BIB_EINVAL, "checkpoint particle %d uses shape %d, which this context does not hold", p, cp.shape);
        const ShapeHost& S = *c->shapes[cp.shape];
        if ((int32_t)(S.rest.size() / 3) != cp.nv || (int32_t)S.tri_area.size() != cp.nt)
            return fail(c, BIB_EINVAL, "shape %d of this context does not match the checkpoint's (%d vertices, %d triangles)",
                        cp.shape, cp.nv, cp.nt);
        if (cp.model < BIB_MODEL_CAPSULE_NEOHOOKEAN || cp.model > BIB_MODEL_SKALAK_BENDING)
            return fail(c, BIB_EINVAL, "corrupt checkpoint particle record");
        ph.shape = cp.shape, ph.model = cp.model, ph.nv = cp.nv, ph.v0 = (int)vtot;
        vtot += cp.nv;
    }
    if (vtot != hd.nvert) return fail(c, BIB_EINVAL, "corrupt checkpoint: vertex count");
    const size_t vb = 3 * (size_t)vtot * sizeof(double);
    std::vector<double> pos(3 * vtot), vel(3 * vtot), frc(3 * vtot), stats(STATS * (size_t)hd.nparts);
    if (vtot && (!F.get(pos.data(), vb) || !F.get(vel.data(), vb) || !F.get(frc.data(), vb) ||
                 !F.get(stats.data(), stats.size() * sizeof(double))))
        return fail(c, BIB_EINVAL, "checkpoint file is truncated");
    uint64_t sum = 0;
    if (fread(&sum, 1, sizeof(sum), F.f) != sizeof(sum) || sum != F.sum.value())
        return fail(c, BIB_EINVAL, "checkpoint checksum mismatch");
    // pass 2: the lattice buffers straight into device memory
    if (fseek(F.f, body_at, SEEK_SET) != 0) return fail(c, BIB_EINVAL, "checkpoint seek failed");
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    bib_status st;
    if ((st = ckpt_get_device(c, F, L->f[hd.cur], pb, buf))) return st;
    if (L->d.fd_walls && (st = ckpt_get_device(c, F, L->wall, wall_bytes(*L), buf))) return st;
    for (int k = 0; k < 2; ++k)
        if ((st = ckpt_get_device(c, F, L->F[k], fb, buf))) return st;
    if (L->phase && (st = ckpt_get_device(c, F, L->phase, (size_t)L->d.stride, buf))) return st;
    if (hd.has_types) {
        std::vector<uint8_t> types((size_t)L->d.n);
        if (!F.get(types.data(), types.size())) return fail(c, BIB_EINVAL, "checkpoint file is truncated");
        for (uint8_t t : types)
            if (t > BIB_CELL_NO_DYNAMICS) return fail(c, BIB_EINVAL, "corrupt checkpoint: cell type %d", (int)t);
        if (!L->celltype) BIB_ALLOC(c, (void**)&L->celltype, (size_t)L->d.n);
        BIB_CUDA(c, cudaMemcpy(L->celltype, types.data(), types.size(), cudaMemcpyHostToDevice));
        L->d.has_types = 1;
    } else if (L->celltype) {
        cudaFree(L->celltype);
        L->celltype = nullptr;
        L->d.has_types = 0;
    }
    for (auto& B : c->batches)  // batch tables hold the lattice description and the particle set
        if (B) B->free_tables();
    L->cur = hd.cur;
    L->fe = hd.fe;
    L->target_clean = hd.target_clean != 0;
    forces_touched(*L);
    L->iteration = hd.iteration;
    // particles: replace the lattice's set, upload, then restore velocities, forces and the
    // per-particle area / volume / centre exactly as saved
    L->parts = std::move(parts);
    L->host_pos = std::move(pos);
    L->host_stats = stats;
    L->particles_dirty = true;
    free_particles(*L);
    L->nvert = 0;
    if ((st = sync_particles(c, *L))) return st;
    if (L->nvert) {
        BIB_CUDA(c, cudaMemcpy(L->vel, vel.data(), vb, cudaMemcpyHostToDevice));
        BIB_CUDA(c, cudaMemcpy(L->force, frc.data(), vb, cudaMemcpyHostToDevice));
    }
    drop_graphs(c, h);
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    return BIB_OK;
}

}  // extern "C"

// ---- the reference's particle files: .plb checkpoints, VTU and lightweight text output ----
namespace {

// the folder part that FileName::setPath gives an output call: "<dir>/", or nothing
std::string folder_prefix(const char* dir) {
    std::string d = dir ? dir : "";
    if (!d.empty() && d.back() != '/') d += '/';
    return d;
}

// FileName of save_checkpoint / load_checkpoint (io/plbFiles.cpp:37-58): the base name
// without folder and extension; the folder and ".plb" come from the call
std::string checkpoint_name(const char* name) {
    std::string n = name ? name : "";
    const size_t sep = n.find_last_of("\\/");
    if (sep != std::string::npos) n = n.substr(sep + 1);
    const size_t dot = n.find_last_of('.');
    if (dot != std::string::npos) n = n.substr(0, dot);
    return n;
}

// positions, velocities, forces (3 per vertex) and STATS per particle on the host
bib_status particle_state(bib_ctx* c, Lattice& L, std::vector<double>& pos, std::vector<double>& vel,
                          std::vector<double>& frc, std::vector<double>& stats) {
    if (L.particles_dirty) {
        pos = L.host_pos;
        vel.assign(pos.size(), 0.0);
        frc.assign(pos.size(), 0.0);
        stats = L.host_stats;
        return BIB_OK;
    }
    const size_t n3 = 3 * (size_t)L.nvert;
    pos.resize(n3);
    vel.resize(n3);
    frc.resize(n3);
    stats.resize(STATS * L.parts.size());
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    if (n3) {
        BIB_CUDA(c, cudaMemcpy(pos.data(), L.pos[L.pcur], n3 * 8, cudaMemcpyDeviceToHost));
        BIB_CUDA(c, cudaMemcpy(vel.data(), L.vel, n3 * 8, cudaMemcpyDeviceToHost));
        BIB_CUDA(c, cudaMemcpy(frc.data(), L.force, n3 * 8, cudaMemcpyDeviceToHost));
    }
    if (!stats.empty())
        BIB_CUDA(c, cudaMemcpy(stats.data(), L.stats, stats.size() * 8, cudaMemcpyDeviceToHost));
    return BIB_OK;
}

bool write_file(const std::string& path, const std::string& bytes, bool binary) {
    FILE* f = fopen(path.c_str(), binary ? "wb" : "w");
    if (!f) return false;
    const bool ok = fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    return fclose(f) == 0 && ok;
}

bool read_file(const std::string& path, std::string& bytes) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    bytes.clear();
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0) bytes.append(buf, n);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

}  // namespace

extern "C" {

bib_status bib_shape_set_tag(bib_ctx* c, int32_t shape, const char* tag) {
    if (!c || !tag || shape < 0 || shape >= (int32_t)c->shapes.size()) return fail(c, BIB_EINVAL, "invalid shape or tag");
    c->shapes[shape]->tag = tag;
    return BIB_OK;
}

bib_status bib_particles_save_plb(bib_ctx* c, int32_t h, const char* dir, const char* name) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    const std::string base = folder_prefix(dir), nm = checkpoint_name(name);
    if (nm.empty()) return fail(c, BIB_EINVAL, "empty checkpoint name");
    std::vector<double> pos, vel, frc, stats;
    bib_status st = particle_state(c, *L, pos, vel, frc, stats);
    if (st) return st;
    // pack everything first: a particle without a reference type leaves no files behind
    std::string body;
    const int64_t np = (int64_t)L->parts.size();
    body.append(reinterpret_cast<const char*>(&np), sizeof(np));
    std::string err;
    for (int64_t p = 0; p < np; ++p) {
        const ParticleHost& ph = L->parts[p];
        PlbParticle pp;
        pp.shape = ph.shape;
        pp.id = p;
        pp.model = ph.model;
        const size_t o = 3 * (size_t)ph.v0, n = 3 * (size_t)ph.nv;
        pp.pos.assign(pos.begin() + o, pos.begin() + o + n);
        pp.vel.assign(vel.begin() + o, vel.begin() + o + n);
        pp.force.assign(frc.begin() + o, frc.begin() + o + n);
        for (int k = 0; k < BIB_P_COUNT; ++k) pp.prm[k] = ph.prm[k];
        if (!plb_pack(body, pp, err)) return fail(c, BIB_EUNSUPPORTED, "particle %lld: %s", (long long)p, err.c_str());
    }
    if (!mkdir_p(base + nm)) return fail(c, BIB_EINVAL, "cannot create the folder %s%s", base.c_str(), nm.c_str());
    const std::string header = std::to_string(np) + "\n1\n" + nm + "/0.plb\n";
    if (!write_file(base + nm + ".plb", header, false))
        return fail(c, BIB_EINVAL, "cannot write the checkpoint header %s%s.plb", base.c_str(), nm.c_str());
    if (!write_file(base + nm + "/0.plb", body, true))
        return fail(c, BIB_EINVAL, "cannot write %s%s/0.plb", base.c_str(), nm.c_str());
    return BIB_OK;
}

bib_status bib_particles_load_plb(bib_ctx* c, int32_t h, const char* dir, const char* name) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    const std::string base = folder_prefix(dir), nm = checkpoint_name(name);
    std::string text;
    if (nm.empty() || !read_file(base + nm + ".plb", text))
        return fail(c, BIB_EINVAL, "cannot read the checkpoint header %s%s.plb", base.c_str(), nm.c_str());
    // header: particle count, file count, then one file name per line (relative to the folder)
    std::vector<std::string> lines;
    {
        size_t at = 0;
        while (at < text.size()) {
            size_t e = text.find('\n', at);
            if (e == std::string::npos) e = text.size();
            lines.push_back(text.substr(at, e - at));
            at = e + 1;
        }
    }
    long long num_particles = -1, num_files = -1;
    if (lines.size() < 2 || sscanf(lines[0].c_str(), "%lld", &num_particles) != 1 ||
        sscanf(lines[1].c_str(), "%lld", &num_files) != 1 || num_particles < 0 || num_files < 0 ||
        (long long)lines.size() < 2 + num_files)
        return fail(c, BIB_EINVAL, "malformed checkpoint header %s%s.plb", base.c_str(), nm.c_str());
    std::vector<int> shape_nv(c->shapes.size());
    for (size_t s = 0; s < c->shapes.size(); ++s) shape_nv[s] = (int)(c->shapes[s]->rest.size() / 3);
    std::vector<PlbParticle> got;
    std::string bytes, err;
    for (long long k = 0; k < num_files; ++k) {
        const std::string path = base + lines[2 + k];
        if (!read_file(path, bytes)) return fail(c, BIB_EINVAL, "cannot read %s", path.c_str());
        const char* it = bytes.data();
        const char* end = it + bytes.size();
        int64_t count = 0;
        if (end - it < 8) return fail(c, BIB_EINVAL, "%s is truncated", path.c_str());
        std::memcpy(&count, it, 8);
        it += 8;
        if (count < 0) return fail(c, BIB_EINVAL, "%s: negative particle count", path.c_str());
        for (int64_t j = 0; j < count; ++j) {
            PlbParticle p;
            if (!plb_unpack(it, end, shape_nv, p, err)) return fail(c, BIB_EINVAL, "%s: %s", path.c_str(), err.c_str());
            got.push_back(std::move(p));
        }
    }
    // this library numbers particles 0 .. n-1: the ids must be exactly those
    const int64_t n = (int64_t)got.size();
    if (num_particles != n)
        return fail(c, BIB_EUNSUPPORTED, "checkpoint holds %lld particles but ids up to %lld", (long long)n, num_particles);
    std::vector<int64_t> slot(n, -1);
    for (int64_t j = 0; j < n; ++j) {
        const int64_t id = got[j].id;
        if (id < 0 || id >= n || slot[id] >= 0)
            return fail(c, BIB_EUNSUPPORTED, "particle ids of the checkpoint are not 0 .. %lld", (long long)(n - 1));
        slot[id] = j;
    }
    std::vector<ParticleHost> parts(n);
    std::vector<double> pos, vel, frc, stats(STATS * (size_t)n);
    int64_t v0 = 0;
    for (int64_t id = 0; id < n; ++id) {
        PlbParticle& p = got[slot[id]];
        if (p.model == BIB_MODEL_RBC_WLCPOW && !(p.prm[BIB_P_VOL_DESIRED] != 0))
            return fail(c, BIB_EINVAL, "particle %lld: vol_desired must be non-zero", (long long)id);
        ParticleHost& ph = parts[id];
        ph.shape = (int)p.shape;
        ph.model = p.model;
        ph.v0 = (int)v0;
        ph.nv = shape_nv[p.shape];
        ph.prm.assign(p.prm, p.prm + BIB_P_COUNT);
        // add_particle maps the centre of mass to the periodic grid (ImmersedBoundaryDynamics.hh:508-525)
        double* s = stats.data() + STATS * id;
        particle_update(*c->shapes[ph.shape], p.pos.data(), s);
        remap_com(L->d, p.pos.data(), ph.nv, s);
        pos.insert(pos.end(), p.pos.begin(), p.pos.end());
        vel.insert(vel.end(), p.vel.begin(), p.vel.end());
        frc.insert(frc.end(), p.force.begin(), p.force.end());
        v0 += ph.nv;
    }
    if (v0 >= ((int64_t)1 << 31)) return fail(c, BIB_EUNSUPPORTED, "too many vertices");
    for (auto& B : c->batches)  // batch tables hold the particle set
        if (B) B->free_tables();
    L->parts = std::move(parts);
    L->host_pos = std::move(pos);
    L->host_stats = std::move(stats);
    L->particles_dirty = true;
    free_particles(*L);
    L->nvert = 0;
    bib_status st = sync_particles(c, *L);
    if (st) return st;
    if (L->nvert) {
        const size_t vb = 3 * (size_t)L->nvert * sizeof(double);
        BIB_CUDA(c, cudaMemcpy(L->vel, vel.data(), vb, cudaMemcpyHostToDevice));
        BIB_CUDA(c, cudaMemcpy(L->force, frc.data(), vb, cudaMemcpyHostToDevice));
    }
    drop_graphs(c, h);
    BIB_CUDA(c, cudaStreamSynchronize(c->stream));
    return BIB_OK;
}

bib_status bib_particle_write_vtu(bib_ctx* c, int32_t h, int32_t pid, const char* path) {
    Lattice* L = get_lattice(c, h);
    if (!L || !path || pid < 0 || pid >= (int32_t)L->parts.size()) return fail(c, BIB_EINVAL, "invalid particle or path");
    std::vector<double> pos, vel, frc, stats;
    bib_status st = particle_state(c, *L, pos, vel, frc, stats);
    if (st) return st;
    const ParticleHost& ph = L->parts[pid];
    const ShapeHost& S = *c->shapes[ph.shape];
    const size_t o = 3 * (size_t)ph.v0;
    if (!write_file(path, vtu_bytes(pos.data() + o, frc.data() + o, ph.nv, S.tri.data(), (int)S.tri_area.size()), true))
        return fail(c, BIB_EINVAL, "cannot write %s", path);
    return BIB_OK;
}

bib_status bib_particles_write_vtu(bib_ctx* c, int32_t h, const char* dir, uint64_t iter) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    std::vector<double> pos, vel, frc, stats;
    bib_status st = particle_state(c, *L, pos, vel, frc, stats);
    if (st) return st;
    const std::string base = folder_prefix(dir);
    if (!base.empty() && !mkdir_p(base)) return fail(c, BIB_EINVAL, "cannot create the folder %s", base.c_str());
    for (size_t p = 0; p < L->parts.size(); ++p) {
        const ParticleHost& ph = L->parts[p];
        const ShapeHost& S = *c->shapes[ph.shape];
        const size_t o = 3 * (size_t)ph.v0;
        const std::string path = base + "obj" + std::to_string(p) + "-" + std::to_string(iter) + ".vtu";
        if (!write_file(path, vtu_bytes(pos.data() + o, frc.data() + o, ph.nv, S.tri.data(), (int)S.tri_area.size()), true))
            return fail(c, BIB_EINVAL, "cannot write %s", path.c_str());
    }
    return BIB_OK;
}

bib_status bib_particles_write_lightweight(bib_ctx* c, int32_t h, const char* dir, uint64_t iter) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    std::vector<double> pos, vel, frc, stats;
    bib_status st = particle_state(c, *L, pos, vel, frc, stats);
    if (st) return st;
    const std::string base = folder_prefix(dir);
    if (!base.empty() && !mkdir_p(base)) return fail(c, BIB_EINVAL, "cannot create the folder %s", base.c_str());
    std::string text = "iteration:" + std::to_string(iter) + "\n";
    for (size_t p = 0; p < L->parts.size(); ++p) {
        const ParticleHost& ph = L->parts[p];
        const double* s = stats.data() + STATS * p;
        text += lightweight_line(c->shapes[ph.shape]->tag, (int64_t)p, pos.data() + 3 * (size_t)ph.v0, ph.nv, s + 2, s[1]);
        text += "\n";
    }
    const std::string path = base + "objsP0-" + std::to_string(iter) + ".txt";
    if (!write_file(path, text, false)) return fail(c, BIB_EINVAL, "cannot write %s", path.c_str());
    return BIB_OK;
}

bib_status bib_lattice_save_plb(bib_ctx* c, int32_t h, const char* dir, const char* name) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    const std::string base = folder_prefix(dir), nm = checkpoint_name(name);
    if (nm.empty()) return fail(c, BIB_EINVAL, "empty checkpoint name");
    const int64_t n = L->d.n;
    std::vector<double> wire((size_t)23 * n);
    bib_status st = bib_lattice_receive(c, h, wire.data(), wire.size() * sizeof(double), BIB_LAYOUT_PALABOS_F64);
    if (st) return st;
    const int64_t bytes = (int64_t)wire.size() * (int64_t)sizeof(double);
    if (!base.empty() && !mkdir_p(base)) return fail(c, BIB_EINVAL, "cannot create the folder %s", base.c_str());
    const std::string xml = plb_lattice_xml(nm + ".dat", L->d.nx, L->d.ny, L->d.nz,
                                            L->d.collision == BIB_COLLISION_BGK_GUO_VOF, bytes);
    if (!write_file(base + nm + ".plb", xml, false))
        return fail(c, BIB_EINVAL, "cannot write %s%s.plb", base.c_str(), nm.c_str());
    if (!write_file(base + nm + ".dat", std::string((const char*)wire.data(), (size_t)bytes), true))
        return fail(c, BIB_EINVAL, "cannot write %s%s.dat", base.c_str(), nm.c_str());
    return BIB_OK;
}

bib_status bib_lattice_load_plb(bib_ctx* c, int32_t h, const char* dir, const char* name) {
    Lattice* L = get_lattice(c, h);
    if (!L) return fail(c, BIB_EINVAL, "invalid lattice handle");
    const std::string base = folder_prefix(dir), nm = checkpoint_name(name);
    std::string xml, err;
    if (nm.empty() || !read_file(base + nm + ".plb", xml))
        return fail(c, BIB_EINVAL, "cannot read %s%s.plb", base.c_str(), nm.c_str());
    PlbLatticeSpec spec;
    if (!plb_lattice_parse(xml, spec, err)) return fail(c, BIB_EINVAL, "%s%s.plb: %s", base.c_str(), nm.c_str(), err.c_str());
    if (spec.dynamic) return fail(c, BIB_EUNSUPPORTED, "checkpoints with dynamic content are not read");
    if (spec.datatype != "double") return fail(c, BIB_EUNSUPPORTED, "data type %s", spec.datatype.c_str());
    if (spec.cell_dim != 22 && spec.cell_dim != 23)
        return fail(c, BIB_EUNSUPPORTED, "cell dimension %d (ForcedD3Q19: 22, ForcedPhaseD3Q19: 23)", spec.cell_dim);
    if (!spec.ordering.empty() && spec.ordering != "zIsFastest")
        return fail(c, BIB_EUNSUPPORTED, "index ordering %s", spec.ordering.c_str());
    const LatticeDesc& d = L->d;
    if (spec.box[0] != 0 || spec.box[1] != d.nx - 1 || spec.box[2] != 0 || spec.box[3] != d.ny - 1 || spec.box[4] != 0 ||
        spec.box[5] != d.nz - 1)
        return fail(c, BIB_EINVAL, "checkpoint lattice is %lld x %lld x %lld", (long long)(spec.box[1] - spec.box[0] + 1),
                    (long long)(spec.box[3] - spec.box[2] + 1), (long long)(spec.box[5] - spec.box[4] + 1));
    // the raw data next to the spec unless its name has a folder; ".dat" unless it has an extension
    std::string dat = spec.file;
    const size_t sep = dat.find_last_of("\\/");
    if (sep == std::string::npos) dat = base + dat;
    if (dat.find('.', sep == std::string::npos ? 0 : sep + 1) == std::string::npos) dat += ".dat";
    std::string raw;
    if (!read_file(dat, raw)) return fail(c, BIB_EINVAL, "cannot read %s", dat.c_str());
    const int per = spec.cell_dim;
    const int64_t n = d.n;
    std::vector<double> wire((size_t)23 * n, 0.0);
    std::vector<uint8_t> seen((size_t)n, 0);
    if (per == 22 && L->phase) {  // no phase in the file: keep the lattice's own
        std::vector<double> ph((size_t)n);
        bib_status st = bib_lattice_get_phase(c, h, ph.data());
        if (st) return st;
        for (int x = 0; x < d.nx; ++x)
            for (int y = 0; y < d.ny; ++y)
                for (int z = 0; z < d.nz; ++z)
                    wire[23 * ((size_t)z + d.nz * ((size_t)y + (size_t)d.ny * x)) + 22] =
                        ph[x + (size_t)d.nx * (y + (size_t)d.ny * z)];
    }
    int64_t start = 0;
    for (size_t b = 0; b < spec.comps.size(); ++b) {
        const std::array<int64_t, 6>& bx = spec.comps[b];
        if (bx[0] < 0 || bx[1] >= d.nx || bx[2] < 0 || bx[3] >= d.ny || bx[4] < 0 || bx[5] >= d.nz || bx[1] < bx[0] ||
            bx[3] < bx[2] || bx[5] < bx[4])
            return fail(c, BIB_EINVAL, "component %zu lies outside the lattice", b);
        const int64_t cells = (bx[1] - bx[0] + 1) * (bx[3] - bx[2] + 1) * (bx[5] - bx[4] + 1);
        const int64_t end = spec.offsets[b];
        if (end - start != cells * per * 8 || end > (int64_t)raw.size())
            return fail(c, BIB_EINVAL, "component %zu: %lld bytes for %lld cells", b, (long long)(end - start), (long long)cells);
        const char* src = raw.data() + start;
        for (int64_t x = bx[0]; x <= bx[1]; ++x)
            for (int64_t y = bx[2]; y <= bx[3]; ++y)
                for (int64_t z = bx[4]; z <= bx[5]; ++z) {
                    const size_t w = (size_t)z + d.nz * ((size_t)y + (size_t)d.ny * x);
                    std::memcpy(&wire[23 * w], src, (size_t)per * 8);
                    src += (size_t)per * 8;
                    seen[w] = 1;
                }
        start = end;
    }
    for (uint8_t v : seen)
        if (!v) return fail(c, BIB_EINVAL, "the components do not cover the lattice");
    return bib_lattice_send(c, h, wire.data(), wire.size() * sizeof(double), BIB_LAYOUT_PALABOS_F64);
}

}  // extern "C"

// ---- RBC shape calibration (progs/common/calibrate_rbc_shape.h) ----
namespace {

// Eigen decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations (the Jacobi method as
// published by J. Kopp, "Efficient numerical diagonalization of hermitian 3x3 matrices", 2008,
// which linalg::diagonalize, fsi/linalg.h:21-138, also follows): eigenvalues w, eigenvectors as
// the columns of Q.  Reads the diagonal and the upper triangle of A and destroys the latter.
void jacobi3(double A[3][3], double Q[3][3], double w[3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Q[i][j] = i == j ? 1.0 : 0.0;
    for (int i = 0; i < 3; ++i) w[i] = A[i][i];
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) off += std::fabs(A[p][q]);
        if (off == 0.0) return;
        const double thresh = sweep < 4 ? 0.2 * off / 9.0 : 0.0;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const double g = 100.0 * std::fabs(A[p][q]);
                if (sweep > 4 && std::fabs(w[p]) + g == std::fabs(w[p]) && std::fabs(w[q]) + g == std::fabs(w[q])) {
                    A[p][q] = 0.0;
                    continue;
                }
                if (!(std::fabs(A[p][q]) > thresh)) continue;
                const double h = w[q] - w[p];
                double t;
                if (std::fabs(h) + g == std::fabs(h)) {
                    t = A[p][q] / h;
                } else {
                    const double theta = 0.5 * h / A[p][q];
                    t = theta < 0.0 ? -1.0 / (std::sqrt(1.0 + theta * theta) - theta)
                                    : 1.0 / (std::sqrt(1.0 + theta * theta) + theta);
                }
                const double cs = 1.0 / std::sqrt(1.0 + t * t), sn = t * cs, z = t * A[p][q];
                A[p][q] = 0.0;
                w[p] -= z;
                w[q] += z;
                // rotate the remaining upper-triangle entries and the eigenvector columns p, q
                auto upper = [&](int a, int b) -> double& { return a < b ? A[a][b] : A[b][a]; };
                for (int r = 0; r < 3; ++r) {
                    if (r == p || r == q) continue;
                    const double ap = upper(r, p), aq = upper(r, q);
                    upper(r, p) = cs * ap - sn * aq;
                    upper(r, q) = sn * ap + cs * aq;
                }
                for (int r = 0; r < 3; ++r) {
                    const double qp = Q[r][p], qq = Q[r][q];
                    Q[r][p] = cs * qp - sn * qq;
                    Q[r][q] = sn * qp + cs * qq;
                }
            }
    }
}

}  // namespace

extern "C" {

bib_status bib_rbc_params(bib_ctx* c, int32_t shape, double shear_modulus, double k_area, double k_bend, double* prm) {
    if (!c || !prm || shape < 0 || shape >= (int32_t)c->shapes.size()) return fail(c, BIB_EINVAL, "invalid shape or output");
    const ShapeHost& S = *c->shapes[shape];
    if (S.link_len.empty()) return fail(c, BIB_EINVAL, "shape has no links");
    double lavg = 0.0;  // average link length
    for (double l : S.link_len) lavg += l;
    lavg /= (double)S.link_len.size();
    for (int k = 0; k < BIB_P_COUNT; ++k) prm[k] = 0.0;
    prm[BIB_P_SHEAR_MODULUS] = shear_modulus;
    prm[BIB_P_L0] = lavg;
    prm[BIB_P_VOL_DESIRED] = S.volume;
    // area constraints: the bulk modulus K = 2 G + k_area_global + k_area_local is k_area
    const double dk = k_area - 2 * shear_modulus;
    prm[BIB_P_K_AREA_GLOBAL] = dk * 0.8;
    prm[BIB_P_K_AREA_LOCAL] = dk * 0.2;
    // radius of the smallest sphere around the origin holding the rest vertices
    // (ParticleShape::compute_bounding_volumes, ParticleShape.hh:361-383)
    double r2 = 0.0;
    const size_t nv = S.rest.size() / 3;
    for (size_t i = 0; i < nv; ++i) {
        const double d2 = S.rest[3 * i] * S.rest[3 * i] + S.rest[3 * i + 1] * S.rest[3 * i + 1] +
                          S.rest[3 * i + 2] * S.rest[3 * i + 2];
        if (d2 > r2) r2 = d2;
    }
    prm[BIB_P_K_VOLUME] = 1000. * shear_modulus / std::sqrt(r2);
    prm[BIB_P_K_BEND] = k_bend;
    // spontaneous angle of a closed triangulation of nv vertices
    const double a = std::sqrt(3.) * ((double)nv - 2.);
    prm[BIB_P_THETA0] = std::acos((a - 5 * M_PI) / (a - 3. * M_PI));
    return BIB_OK;
}

bib_status bib_rbc_shrink_volume(bib_ctx* c, int32_t shape, const double* params, double vol_final, int64_t n_it,
                                 double damping, double* pos_out, double* damping_out) {
    if (!c || !params || !pos_out || shape < 0 || shape >= (int32_t)c->shapes.size())
        return fail(c, BIB_EINVAL, "invalid shape or argument");
    if (n_it < 1 || n_it > ((int64_t)1 << 40) || !(damping > 0) || !std::isfinite(damping) || !(vol_final > 0) ||
        !std::isfinite(vol_final) || !(params[BIB_P_VOL_DESIRED] != 0))
        return fail(c, BIB_EINVAL, "need n_it >= 1, damping > 0, vol_final > 0, vol_desired != 0");
    const ShapeHost& S = *c->shapes[shape];
    const int nv = (int)(S.rest.size() / 3);
    // a holder of the one particle: no lattice buffers, no periodic remap
    Lattice L;
    L.d.nx = L.d.ny = L.d.nz = 1;
    L.d.n = 1;
    L.d.stride = 128;
    L.storage = BIB_STORAGE_F64;
    L.ib = IbDesc{BIB_DIRAC_ROMA, BIB_SPREAD_ATOMIC, -1.0};
    ParticleHost ph;
    ph.shape = shape;
    ph.model = BIB_MODEL_RBC_WLCPOW;
    ph.v0 = 0;
    ph.nv = nv;
    ph.prm.assign(params, params + BIB_P_COUNT);
    L.parts.push_back(ph);
    long long* iter = nullptr;
    BIB_ALLOC(c, (void**)&iter, sizeof(long long));
    bib_status st = BIB_OK;
    cudaStream_t s = c->stream;
    for (int attempt = 0;; ++attempt) {
        if (attempt == 64) {
            st = fail(c, BIB_ENAN, "the relaxation diverged up to damping %g", damping);
            break;
        }
        // the particle as constructed on the shape: rest positions, the shape's area and volume,
        // zero velocities, then its forces (calibrate_rbc_shape.h:20)
        double st5[STATS];
        particle_update(S, S.rest.data(), st5);
        st5[0] = S.area;
        st5[1] = S.volume;
        L.host_pos = S.rest;
        L.host_stats.assign(st5, st5 + STATS);
        L.particles_dirty = true;
        if ((st = sync_particles(c, L))) break;
        if (cudaMemsetAsync(iter, 0, sizeof(long long), s) != cudaSuccess) {
            st = fail(c, BIB_ECUDA, "memset failed");
            break;
        }
        launch_membrane_forces(L, s);
        bool diverged = false;
        for (int64_t it = 0; it <= 2 * n_it; ++it) {
            launch_rbc_relax(L, damping, iter, n_it, S.volume, vol_final, s);
            launch_particle_update(L, s);
            L.pcur = 1 - L.pcur;
            launch_membrane_forces(L, s);
            if ((it & 255) == 255 || it == 2 * n_it) {  // NaN persists: checking a chunk's end is enough
                double area = 0;
                if (cudaMemcpyAsync(&area, L.stats, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                    cudaStreamSynchronize(s) != cudaSuccess) {
                    st = fail(c, BIB_ECUDA, "calibration step failed: %s", cudaGetErrorString(cudaGetLastError()));
                    break;
                }
                if (area != area) {
                    diverged = true;
                    break;
                }
            }
        }
        if (st) break;
        if (!diverged) {
            if (cudaMemcpy(pos_out, L.pos[L.pcur], 3 * (size_t)nv * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
                st = fail(c, BIB_ECUDA, "download failed");
            break;
        }
        damping *= 2.;
    }
    free_particles(L);
    cudaFree(iter);
    if (!st && damping_out) *damping_out = damping;
    return st;
}

bib_status bib_align_minor_axis(bib_ctx* c, int32_t shape, double* pos, const double* dir) {
    if (!c || !pos || !dir || shape < 0 || shape >= (int32_t)c->shapes.size())
        return fail(c, BIB_EINVAL, "invalid shape or argument");
    const ShapeHost& S = *c->shapes[shape];
    const int nv = (int)(S.rest.size() / 3);
    double st[STATS];
    particle_update(S, pos, st);
    const double* com = st + 2;
    // tensor of gyration (DeformableParticle3D.hh:111-125)
    double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int v = 0; v < nv; ++v)
        for (int i = 0; i < 3; ++i)
            for (int j = i; j < 3; ++j) A[i][j] += (pos[3 * v + i] - com[i]) * (pos[3 * v + j] - com[j]);
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) A[i][j] /= nv;
    double Q[3][3], w[3];
    jacobi3(A, Q, w);
    // minor axis: the eigenvector of the smallest |eigenvalue| (DeformableParticle3D.hh:85-99)
    const double a0 = std::fabs(w[0]), a1 = std::fabs(w[1]), a2 = std::fabs(w[2]);
    const int k = (a0 < a1 && a0 < a2) ? 0 : (a1 < a2) ? 1 : 2;
    double d[3] = {Q[0][k], Q[1][k], Q[2][k]};
    const double dn = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (double& x : d) x /= dn;
    // rotate_to_align_vectors (DeformableParticle3D.hh:128-144) about the centre of mass
    double ax[3] = {d[1] * dir[2] - d[2] * dir[1], d[2] * dir[0] - d[0] * dir[2], d[0] * dir[1] - d[1] * dir[0]};
    const double an = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    const double pn = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (!(pn > 0)) return fail(c, BIB_EINVAL, "zero direction");
    if (an == 0.0) return BIB_OK;  // already aligned (the reference divides by zero here)
    const double angle = std::asin(an / (std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * pn));
    for (double& x : ax) x /= an;
    if (dir[0] * d[0] + dir[1] * d[1] + dir[2] * d[2] < 0)
        for (double& x : ax) x = -x;
    const double sh = std::sin(angle / 2), q0 = std::cos(angle / 2), q1 = sh * ax[0], q2 = sh * ax[1], q3 = sh * ax[2];
    const double R[3][3] = {{1 - 2 * (q2 * q2 + q3 * q3), 2 * (q1 * q2 - q0 * q3), 2 * (q0 * q2 + q1 * q3)},
                            {2 * (q1 * q2 + q0 * q3), 1 - 2 * (q1 * q1 + q3 * q3), 2 * (q2 * q3 - q0 * q1)},
                            {2 * (q1 * q3 - q0 * q2), 2 * (q0 * q1 + q2 * q3), 1 - 2 * (q1 * q1 + q2 * q2)}};
    // Transform: translate(-com), rotate(R), translate(com), applied as a 3 x 4 affine map
    double m[3][4];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) m[i][j] = R[i][j];
        m[i][3] = R[i][0] * -com[0] + R[i][1] * -com[1] + R[i][2] * -com[2] + com[i];
    }
    for (int v = 0; v < nv; ++v) {
        const double x = pos[3 * v], y = pos[3 * v + 1], z = pos[3 * v + 2];
        for (int i = 0; i < 3; ++i) pos[3 * v + i] = x * m[i][0] + y * m[i][1] + z * m[i][2] + m[i][3];
    }
    return BIB_OK;
}

}  // extern "C"

// ParticleShape::compute_properties' moment of inertia about the origin (ParticleShape.hh:254-356)
static void shape_inertia_origin(const ShapeHost& S, double* I) {
    double in[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int nt = (int)(S.tri.size() / 3);
    const double* pos = S.rest.data();
    for (int t = 0; t < nt; ++t) {
        const double* v0 = pos + 3 * S.tri[3 * t];
        const double* v1 = pos + 3 * S.tri[3 * t + 1];
        const double* v2 = pos + 3 * S.tri[3 * t + 2];
        const V3d N = crs(V3d{v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]}, V3d{v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]});
        double f2[3], f3[3], g0[3], g1[3], g2[3];
        for (int d = 0; d < 3; ++d) {
            const double tmp0 = v0[d] + v1[d];
            const double f1 = tmp0 + v2[d];
            const double tmp1 = v0[d] * v0[d];
            const double tmp2 = tmp1 + v1[d] * tmp0;
            f2[d] = tmp2 + v2[d] * f1;
            f3[d] = v0[d] * tmp1 + v1[d] * tmp2 + v2[d] * f2[d];
            g0[d] = f2[d] + v0[d] * (f1 + v0[d]);
            g1[d] = f2[d] + v1[d] * (f1 + v1[d]);
            g2[d] = f2[d] + v2[d] * (f1 + v2[d]);
        }
        in[4] += N.x * f3[0];
        in[5] += N.y * f3[1];
        in[6] += N.z * f3[2];
        in[7] += N.x * (v0[1] * g0[0] + v1[1] * g1[0] + v2[1] * g2[0]);
        in[8] += N.y * (v0[2] * g0[1] + v1[2] * g1[1] + v2[2] * g2[1]);
        in[9] += N.z * (v0[0] * g0[2] + v1[0] * g1[2] + v2[0] * g2[2]);
    }
    for (int k = 4; k <= 6; ++k) in[k] *= (double)(1.0 / 60.0);
    for (int k = 7; k <= 9; ++k) in[k] *= (double)(1.0 / 120.0);
    I[0] = in[5] + in[6];
    I[1] = -in[7];
    I[2] = -in[9];
    I[3] = I[1];
    I[4] = in[4] + in[6];
    I[5] = -in[8];
    I[6] = I[2];
    I[7] = I[5];
    I[8] = in[4] + in[5];
}

// Device buffers of one call, freed when it returns.
struct CallBuffers {
    std::vector<void*> p;
    ~CallBuffers() {
        for (void* q : p) cudaFree(q);
    }
    bool get(bib_ctx* c, void** out, size_t bytes) {
        if (dev_malloc(c, out, std::max<size_t>(bytes, 16)) != cudaSuccess) {
            cudaGetLastError();
            *out = nullptr;
            return false;
        }
        p.push_back(*out);
        return true;
    }
};

extern "C" {

bib_status bib_grow_particles(bib_ctx* c, const bib_growth* g, int32_t n, const int32_t* shape, double* com,
                              double* quat, double* pos_out, double* force_out) {
    if (!c || !g || n < 0 || (n > 0 && (!shape || !com || !quat))) return fail(c, BIB_EINVAL, "invalid argument");
    for (int a = 0; a < 3; ++a)
        if (g->box[2 * a + 1] - g->box[2 * a] < 1 || g->box[2 * a + 1] - g->box[2 * a] > (1 << 20))
            return fail(c, BIB_EINVAL, "box extents must be in [2, 2^20 + 1]");
    const double vals[] = {g->min_dist, g->strength, g->initial_scale, g->density, g->damping,
                           g->wall[0], g->wall[1], g->wall[2]};
    for (double v : vals)
        if (!std::isfinite(v)) return fail(c, BIB_EINVAL, "growth parameters must be finite");
    if (!(g->min_dist > 0 && g->min_dist <= 1.0)) return fail(c, BIB_EINVAL, "min_dist must be in (0, 1]");
    if (!(g->initial_scale > 0) || !(g->density > 0) || g->n_it < 1 || g->rescale_every < 1 || g->it_end < 0 ||
        g->it_end > g->n_it + 1 || (g->has_wall && !(g->wall[2] > 0)))
        return fail(c, BIB_EINVAL, "need initial_scale, density > 0, n_it, rescale_every >= 1, 0 <= it_end <= n_it + 1");
    // the shapes in use and the vertex ranges of the particles
    std::vector<int> local(c->shapes.size(), -1), used;
    std::vector<int> pshape(n), pv0(n);
    int64_t nvert = 0;
    for (int k = 0; k < n; ++k) {
        if (shape[k] < 0 || shape[k] >= (int32_t)c->shapes.size()) return fail(c, BIB_EINVAL, "invalid shape %d", shape[k]);
        if (local[shape[k]] < 0) {
            local[shape[k]] = (int)used.size();
            used.push_back(shape[k]);
        }
        pshape[k] = local[shape[k]];
        pv0[k] = (int)nvert;
        nvert += (int64_t)(c->shapes[shape[k]]->rest.size() / 3);
        for (int d = 0; d < 3; ++d)
            if (!std::isfinite(com[3 * k + d])) return fail(c, BIB_EINVAL, "non-finite centre");
        for (int d = 0; d < 4; ++d)
            if (!std::isfinite(quat[4 * k + d])) return fail(c, BIB_EINVAL, "non-finite orientation");
    }
    if (nvert > (1 << 28)) return fail(c, BIB_EINVAL, "too many vertices");
    const int ns = (int)used.size();
    std::vector<int> snv(ns), sv0(ns);
    std::vector<double> verts, vol(ns), inertia(9 * (size_t)ns);
    for (int s = 0; s < ns; ++s) {
        const ShapeHost& S = *c->shapes[used[s]];
        snv[s] = (int)(S.rest.size() / 3);
        sv0[s] = (int)(verts.size() / 3);
        verts.insert(verts.end(), S.rest.begin(), S.rest.end());
        vol[s] = S.volume;
        shape_inertia_origin(S, &inertia[9 * (size_t)s]);
    }
    std::vector<int> owner((size_t)nvert);
    for (int k = 0; k < n; ++k)
        for (int i = 0; i < snv[pshape[k]]; ++i) owner[(size_t)pv0[k] + i] = k;
    const int per[3] = {g->periodic[0] ? 1 : 0, g->periodic[1] ? 1 : 0, g->periodic[2] ? 1 : 0};
    if (ref_grid_cells(g->box) > kMaxRefGridCells) return fail(c, BIB_EINVAL, "box too large for the collision grid");
    const RefGrid grid = ref_grid(g->box, per, g->min_dist, (int)nvert);
    CallBuffers B;
    GrowthView G;
    RefGridBuffers R;
    R.bits = ref_grid_bits(grid.ncell);
    R.temp_bytes = ref_grid_temp_bytes((int)nvert, R.bits);
    int *d_shape, *d_pv0, *d_snv, *d_sv0, *d_owner;
    double *d_verts, *d_vol, *d_inertia, *d_state, *d_pos, *d_force, *d_torque;
    const size_t np = (size_t)std::max(n, 1);
    const bool ok = B.get(c, (void**)&d_shape, np * sizeof(int)) && B.get(c, (void**)&d_pv0, np * sizeof(int)) &&
                    B.get(c, (void**)&d_snv, ns * sizeof(int)) && B.get(c, (void**)&d_sv0, ns * sizeof(int)) &&
                    B.get(c, (void**)&d_owner, nvert * sizeof(int)) &&
                    B.get(c, (void**)&d_verts, verts.size() * sizeof(double)) &&
                    B.get(c, (void**)&d_vol, ns * sizeof(double)) &&
                    B.get(c, (void**)&d_inertia, 9 * ns * sizeof(double)) &&
                    B.get(c, (void**)&d_state, 13 * np * sizeof(double)) &&
                    B.get(c, (void**)&d_pos, 3 * nvert * sizeof(double)) &&
                    B.get(c, (void**)&d_force, 3 * nvert * sizeof(double)) &&
                    B.get(c, (void**)&d_torque, 3 * nvert * sizeof(double)) &&
                    B.get(c, (void**)&R.keys[0], nvert * sizeof(uint32_t)) &&
                    B.get(c, (void**)&R.keys[1], nvert * sizeof(uint32_t)) &&
                    B.get(c, (void**)&R.ids[0], nvert * sizeof(uint32_t)) &&
                    B.get(c, (void**)&R.ids[1], nvert * sizeof(uint32_t)) &&
                    B.get(c, (void**)&R.posf, nvert * sizeof(float4)) &&
                    B.get(c, (void**)&R.start, ((size_t)grid.ncell + 1) * sizeof(int)) &&
                    B.get(c, (void**)&R.end, ((size_t)grid.ncell + 1) * sizeof(int)) && B.get(c, &R.temp, R.temp_bytes);
    if (!ok) return fail(c, BIB_ENOMEM, "device allocation for the growth stage failed");
    std::vector<double> state(13 * np, 0.0);  // com, quat, vel, omega
    for (int k = 0; k < n; ++k) {
        for (int d = 0; d < 3; ++d) state[3 * (size_t)k + d] = com[3 * k + d];
        for (int d = 0; d < 4; ++d) state[3 * np + 4 * (size_t)k + d] = quat[4 * k + d];
    }
    cudaStream_t st = c->stream;
    BIB_CUDA(c, cudaMemcpyAsync(d_shape, pshape.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_pv0, pv0.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_snv, snv.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_sv0, sv0.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_owner, owner.data(), nvert * sizeof(int), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_verts, verts.data(), verts.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_vol, vol.data(), ns * sizeof(double), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_inertia, inertia.data(), 9 * ns * sizeof(double), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_state, state.data(), 13 * np * sizeof(double), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemsetAsync(d_force, 0, 3 * nvert * sizeof(double), st));
    BIB_CUDA(c, cudaMemsetAsync(R.keys[1], 0, nvert * sizeof(uint32_t), st));
    BIB_CUDA(c, cudaMemsetAsync(R.start, 0, ((size_t)grid.ncell + 1) * sizeof(int), st));
    BIB_CUDA(c, cudaMemsetAsync(R.end, 0, ((size_t)grid.ncell + 1) * sizeof(int), st));
    G.np = n;
    G.shape = d_shape;
    G.part_v0 = d_pv0;
    G.shape_nv = d_snv;
    G.shape_v0 = d_sv0;
    G.verts = d_verts;
    G.volume = d_vol;
    G.inertia = d_inertia;
    G.com = d_state;
    G.quat = d_state + 3 * np;
    G.vel = d_state + 7 * np;
    G.omega = d_state + 10 * np;
    G.pos = d_pos;
    G.force = d_force;
    G.torque = d_torque;
    G.density = g->density;
    G.damping = g->damping;
    for (int a = 0; a < 3; ++a) {
        G.per[a] = per[a];
        G.x0[a] = (double)g->box[2 * a] - 0.5;
        G.L[a] = (double)(g->box[2 * a + 1] - g->box[2 * a] + 1);
        G.Linv[a] = 1. / G.L[a];
    }
    const PotentialDev pot{BIB_POTENTIAL_SPRING, g->min_dist, 0.0, g->strength};
    const double wall[3] = {g->wall[0], g->wall[1], g->wall[2]};
    // the scales of the rescale iterations (create_particles.h:132-147), in the driver's arithmetic
    std::vector<double> scales((size_t)(g->it_end > 0 ? (g->it_end - 1) / g->rescale_every + 1 : 1));
    for (size_t r = 0; r < scales.size(); ++r) {
        const double fraction = (double)((int64_t)r * g->rescale_every) / (double)g->n_it;
        scales[r] = g->initial_scale + (1. - g->initial_scale) * fraction;
    }
    double* d_scales;
    long long* d_it;
    double* d_scale_now;
    if (!B.get(c, (void**)&d_scales, scales.size() * sizeof(double)) || !B.get(c, (void**)&d_it, sizeof(long long)) ||
        !B.get(c, (void**)&d_scale_now, sizeof(double)))
        return fail(c, BIB_ENOMEM, "device allocation for the growth stage failed");
    const long long zero = 0;
    BIB_CUDA(c, cudaMemcpyAsync(d_scales, scales.data(), scales.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_it, &zero, sizeof(long long), cudaMemcpyHostToDevice, st));
    BIB_CUDA(c, cudaMemcpyAsync(d_scale_now, &g->initial_scale, sizeof(double), cudaMemcpyHostToDevice, st));
    G.it = d_it;
    G.scales = d_scales;
    G.every = g->rescale_every;
    G.scale_now = d_scale_now;
    launch_rigid_nodes(G, g->initial_scale, st);
    auto iteration = [&]() {
        launch_rigid_rescale(G, st);
        launch_ref_grid_forces(grid, R, pot, d_pos, d_owner, d_force, true, g->has_wall ? wall : nullptr, st);
        launch_rigid_move(G, st);
    };
    // a block of iterations captured once and replayed: the schedule lives in device memory
    constexpr int kBlock = 16;
    int64_t done = 0;
    if (g->it_end >= 2 * kBlock) {
        BIB_CUDA(c, cudaStreamSynchronize(st));
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        BIB_CUDA(c, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kBlock; ++k) iteration();
        const cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (ec != cudaSuccess) return fail(c, BIB_ECUDA, "growth graph capture failed: %s", cudaGetErrorString(ec));
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return fail(c, BIB_ECUDA, "growth graph: %s", cudaGetErrorString(ei));
        cudaError_t el = cudaSuccess;
        for (; done + kBlock <= g->it_end && el == cudaSuccess; done += kBlock) el = cudaGraphLaunch(exec, st);
        cudaGraphExecDestroy(exec);
        if (el != cudaSuccess) return fail(c, BIB_ECUDA, "growth graph launch: %s", cudaGetErrorString(el));
    }
    for (; done < g->it_end; ++done) iteration();
    BIB_CHECK_LAUNCH(c);
    BIB_CUDA(c, cudaMemcpyAsync(state.data(), d_state, 7 * np * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (pos_out) BIB_CUDA(c, cudaMemcpyAsync(pos_out, d_pos, 3 * nvert * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (force_out) BIB_CUDA(c, cudaMemcpyAsync(force_out, d_force, 3 * nvert * sizeof(double), cudaMemcpyDeviceToHost, st));
    BIB_CUDA(c, cudaStreamSynchronize(st));
    for (int k = 0; k < n; ++k) {
        for (int d = 0; d < 3; ++d) com[3 * k + d] = state[3 * (size_t)k + d];
        for (int d = 0; d < 4; ++d) quat[4 * k + d] = state[3 * np + 4 * (size_t)k + d];
    }
    return BIB_OK;
}

bib_status bib_place_particle(bib_ctx* c, int32_t shape, const double* xyz, const double* com, const double* quat,
                              double* out) {
    if (!c || !com || !quat || !out || shape < 0 || shape >= (int32_t)c->shapes.size())
        return fail(c, BIB_EINVAL, "invalid shape or argument");
    const ShapeHost& S = *c->shapes[shape];
    const int nv = (int)(S.rest.size() / 3);
    const double* v = xyz ? xyz : S.rest.data();
    double st[STATS];
    particle_update(S, v, st);
    const double* cm = st + 2;
    const double* q = quat;
    const double R[3][3] = {{1 - 2 * (q[2] * q[2] + q[3] * q[3]), 2 * (q[1] * q[2] - q[0] * q[3]), 2 * (q[0] * q[2] + q[1] * q[3])},
                            {2 * (q[1] * q[2] + q[0] * q[3]), 1 - 2 * (q[1] * q[1] + q[3] * q[3]), 2 * (q[2] * q[3] - q[0] * q[1])},
                            {2 * (q[1] * q[3] - q[0] * q[2]), 2 * (q[0] * q[1] + q[2] * q[3]), 1 - 2 * (q[1] * q[1] + q[2] * q[2])}};
    // Transform().translate(-c).rotate(R).translate(com) as the 3 x 4 map it builds
    double m3[3];
    for (int i = 0; i < 3; ++i) m3[i] = R[i][0] * -cm[0] + R[i][1] * -cm[1] + R[i][2] * -cm[2] + com[i];
    for (int k = 0; k < nv; ++k) {
        const double x = v[3 * k], y = v[3 * k + 1], z = v[3 * k + 2];
        for (int i = 0; i < 3; ++i) out[3 * k + i] = x * R[i][0] + y * R[i][1] + z * R[i][2] + m3[i];
    }
    return BIB_OK;
}

}  // extern "C"
