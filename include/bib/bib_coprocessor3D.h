/* Palabos co-processor backed by biblbm_gb300.
 *
 * plb::BibCoProcessor3D implements CoProcessor3D<double> (src/coProcessors/coProcessor3D.h:57-115
 * of the reference) on top of the C ABI of bib/bib.h, so that MultiBlockLattice3D::collideAndStream
 * (src/multiBlock/multiBlockLattice3D.hh:308-322) runs the blocks attributed to the co-processor on
 * the GPU.  Header only, C++98 (the reference builds with -std=gnu++98); include it after
 * coProcessors/coProcessor3D.h (palabos3D.h includes that) and link libbib_gb300.so.
 *
 * The interface's contract, as the reference states it, and how it maps:
 *   - addDomain(nx, ny, nz, omega, handle): a block of nx x ny x nz cells.  Palabos passes the
 *     block with its envelope (SmartBulk3D::computeEnvelope, coProcessorCommunication3D.hh:111-115).
 *     The result of collideAndStream is undefined in the outer one-cell layer
 *     (coProcessor3D.h:105-107) and Palabos overwrites that layer (the envelope) from the
 *     neighbouring blocks; this adapter wraps the layer periodically, which is one admissible
 *     choice for it.
 *   - send / receive: cell-major bytes, the 19 populations of a cell fastest, then z, y, x
 *     (coProcessor3D.h:80-91), as DataTransfer::send / receive of modif::staticVariables writes
 *     them: f-bar = f - t_i.  A D3Q19 block gives 19 doubles per cell (BIB_LAYOUT_COPROCESSOR_F64);
 *     a ForcedPhaseD3Q19 block 23 (the populations, the force and the phase:
 *     BIB_LAYOUT_PALABOS_F64).  The layout is taken from the byte count of the first send.  Only
 *     whole blocks are transferred (transferToCoProcessors sends getBoundingBox()).
 *   - collideAndStream(handle): one BGK step (BGK with Guo forcing when constructed with
 *     BIB_COLLISION_BGK_GUO_VOF), blocking, as the interface requires.
 *   - return codes: 1 = success, 0 = failure (BIB_OK -> 1, any negative bib_status -> 0); the
 *     library's message is available through bib_last_error(context(), ...).
 *
 * Storage: BIB_STORAGE_F64 (default) keeps the reference's FP64 arithmetic; BIB_STORAGE_F32 /
 * BIB_STORAGE_F16 store deviations f - t_i at reduced precision and collide in FP32.
 *
 * To use it, make it the singleton of global::defaultCoProcessor3D<double>()
 * (coProcessor3D.h:176-187).  Not thread-safe: one host thread drives a context. */
#ifndef BIB_COPROCESSOR3D_H
#define BIB_COPROCESSOR3D_H

#include <cstring>
#include <map>
#include <vector>

#include "bib/bib.h"

namespace plb {

class BibCoProcessor3D : public CoProcessor3D<double> {
public:
    explicit BibCoProcessor3D(int device = 0, int storage = BIB_STORAGE_F64, int collision = BIB_COLLISION_BGK)
        : ctx_(0), storage_(storage), collision_(collision) {
        bib_config cfg;
        std::memset(&cfg, 0, sizeof(cfg));
        cfg.device = device;
        if (bib_create(&cfg, &ctx_) != BIB_OK) ctx_ = 0;
    }
    virtual ~BibCoProcessor3D() {
        if (ctx_) bib_destroy(ctx_);
    }

    /* CoProcessor3D::addDomain, coProcessor3D.h:69-74 */
    virtual int addDomain(plint nx, plint ny, plint nz, double omega, int& domainHandle) {
        if (!ctx_) return 0;
        bib_lattice_params p;
        if (bib_coprocessor_domain_params(omega, storage_, collision_, &p) != BIB_OK) return 0;
        int32_t h = -1;
        if (bib_lattice_add_domain(ctx_, (int64_t)nx, (int64_t)ny, (int64_t)nz, &p, &h) != BIB_OK) return 0;
        Domain d;
        d.nx = nx;
        d.ny = ny;
        d.nz = nz;
        d.per = 0;
        domains_[h] = d;
        domainHandle = h;
        return 1;
    }

    /* CoProcessor3D::send, coProcessor3D.h:76-91: the whole block, cell-major */
    virtual int send(int domainHandle, Box3D const& subDomain, std::vector<char> const& data) {
        std::map<int, Domain>::iterator it = domains_.find(domainHandle);
        if (!ctx_ || it == domains_.end() || !whole(it->second, subDomain) || data.empty()) return 0;
        Domain& d = it->second;
        const size_t cells = (size_t)d.nx * (size_t)d.ny * (size_t)d.nz;
        int per = 0;
        if (data.size() == cells * 19 * sizeof(double)) per = 19;
        else if (data.size() == cells * 23 * sizeof(double)) per = 23;
        else return 0;
        const int32_t layout = per == 19 ? BIB_LAYOUT_COPROCESSOR_F64 : BIB_LAYOUT_PALABOS_F64;
        if (bib_lattice_send(ctx_, domainHandle, &data[0], data.size(), layout) != BIB_OK) return 0;
        d.per = per;
        return 1;
    }

    /* CoProcessor3D::receive, coProcessor3D.h:93-101: resizes data to the block, in the layout
     * of the last send (19 doubles per cell before any send) */
    virtual int receive(int domainHandle, Box3D const& subDomain, std::vector<char>& data) const {
        std::map<int, Domain>::const_iterator it = domains_.find(domainHandle);
        if (!ctx_ || it == domains_.end() || !whole(it->second, subDomain)) return 0;
        const Domain& d = it->second;
        const int per = d.per ? d.per : 19;
        data.resize((size_t)d.nx * (size_t)d.ny * (size_t)d.nz * (size_t)per * sizeof(double));
        const int32_t layout = per == 19 ? BIB_LAYOUT_COPROCESSOR_F64 : BIB_LAYOUT_PALABOS_F64;
        return bib_lattice_receive(ctx_, domainHandle, &data[0], data.size(), layout) == BIB_OK ? 1 : 0;
    }

    /* CoProcessor3D::collideAndStream, coProcessor3D.h:103-113: blocking */
    virtual int collideAndStream(int domainHandle) {
        if (!ctx_ || domains_.find(domainHandle) == domains_.end()) return 0;
        if (bib_lattice_collide_and_stream(ctx_, domainHandle, 1) != BIB_OK) return 0;
        return bib_sync(ctx_) == BIB_OK ? 1 : 0;
    }

    /* the library context (for bib_last_error, tuning, checkpoints); null if the device could
     * not be opened, in which case every call returns 0 */
    bib_ctx* context() const { return ctx_; }

private:
    struct Domain {
        plint nx, ny, nz;
        int per;  /* doubles per cell of the last send, 0 before it */
    };
    static bool whole(const Domain& d, Box3D const& b) {
        return b.x0 == 0 && b.y0 == 0 && b.z0 == 0 && b.x1 == d.nx - 1 && b.y1 == d.ny - 1 && b.z1 == d.nz - 1;
    }
    BibCoProcessor3D(BibCoProcessor3D const&);
    BibCoProcessor3D& operator=(BibCoProcessor3D const&);

    bib_ctx* ctx_;
    int storage_, collision_;
    std::map<int, Domain> domains_;
};

}  // namespace plb

#endif  // BIB_COPROCESSOR3D_H
