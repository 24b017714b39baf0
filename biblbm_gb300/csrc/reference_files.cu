// The reference's on-disk particle formats, host side (no device code in this file).
//
//   .plb particle checkpoint  ImmersedBoundaryDynamics3D::save_checkpoint / load_checkpoint
//                             (src/fsi/ImmersedBoundaryDynamics_io.hh:17-159): a text header
//                             <dir>/<name>.plb with the particle count, the file count and one
//                             file name per rank, and per rank a binary file <dir>/<name>/<r>.plb
//                             holding an int64 particle count followed by each particle's pack.
//   particle pack             raw native (little-endian) bytes, in this order:
//                             ParticleBase3D::pack (ParticleBase.hh:218-224): int64 type id,
//                             int64 shape id, int64 particle id, one byte should_voxelize;
//                             DeformableParticle3D::pack (DeformableParticle3D.hh:277-287): per
//                             vertex pos, vel, force as 3 doubles each; then the model's own
//                             part: DeformableCapsuleParticle::pack (DeformableCapsule.hh:217-223)
//                             int32 shear model (0 Skalak, 1 NeoHookean) and CapsuleParameters::pack
//                             (DeformableCapsule.hh:21-29) C, kb, nu_s, G; RBCParticle::pack
//                             (RBCParticle.hh:344-350) RBCParameters::pack (RBCParticle.hh:93-105)
//                             L0, shear_modulus, k_area_global, k_area_local, k_bend, k_volume,
//                             theta0, vol_desired.
//   VTU particle output       ParticleBase3D::write_vtk (ParticleBase.hh:270-390): an XML
//                             UnstructuredGrid with raw appended data (UInt32 block sizes, Float32
//                             positions and forces, Int32 triangles, offsets and cell types).
//   lightweight text output   DeformableParticle3D::write_lightweight (DeformableParticle3D.hh:
//                             318-333): tag:id:centre:gyration tensor (upper triangle):volume,
//                             default stream formatting.
//   lattice checkpoint        parallelIO::save / load with static content (io/multiBlockWriter3D.cpp:
//                             53-137, 201-213, 273-310; io/multiBlockReader3D.cpp:135-268): an XML
//                             spec <name>.plb listing the lattice's blocks ("components", inclusive
//                             boxes) and the end offset of each block's bytes in the raw file
//                             <name>.dat; a block's bytes are its cells x-major with z fastest, each
//                             cell its 19 populations f-bar then its external scalars
//                             (BlockLattice3D::send, blockLattice3D.hh:671-689), as doubles.
#include "bib_internal.h"

#include <sys/stat.h>
#include <cerrno>
#include <cstring>
#include <sstream>

namespace bib {

namespace {

template <class V>
void put(std::string& out, const V& v) {
    out.append(reinterpret_cast<const char*>(&v), sizeof(V));
}

template <class V>
bool get(const char*& it, const char* end, V& v) {
    if (end - it < (ptrdiff_t)sizeof(V)) return false;
    std::memcpy(&v, it, sizeof(V));
    it += sizeof(V);
    return true;
}

// parameter order of the capsule and RBC parameter packs, as BIB_P_* indices
constexpr int kCapsulePack[4] = {BIB_P_C, BIB_P_KB, BIB_P_NU_S, BIB_P_G};
constexpr int kRbcPack[8] = {BIB_P_L0, BIB_P_SHEAR_MODULUS, BIB_P_K_AREA_GLOBAL, BIB_P_K_AREA_LOCAL,
                             BIB_P_K_BEND, BIB_P_K_VOLUME, BIB_P_THETA0, BIB_P_VOL_DESIRED};
constexpr int32_t kShearSkalak = 0, kShearNeoHookean = 1;  // enum ShearModel, DeformableCapsule.h:39

}  // namespace

bool plb_pack(std::string& out, const PlbParticle& p, std::string& err) {
    int64_t type;
    if (p.model == BIB_MODEL_CAPSULE_NEOHOOKEAN || p.model == BIB_MODEL_CAPSULE_SKALAK) {
        type = kPlbTypeCapsule;
    } else if (p.model == BIB_MODEL_RBC_WLCPOW) {
        type = kPlbTypeRbc;
    } else {
        err = "particle model has no particle type in the reference's format";
        return false;
    }
    const size_t nv = p.pos.size() / 3;
    if (p.vel.size() != 3 * nv || p.force.size() != 3 * nv) {
        err = "vertex arrays of different lengths";
        return false;
    }
    put(out, type);
    put(out, p.shape);
    put(out, p.id);
    put(out, (bool)p.voxelize);
    for (size_t i = 0; i < nv; ++i) {
        for (int a = 0; a < 3; ++a) put(out, p.pos[3 * i + a]);
        for (int a = 0; a < 3; ++a) put(out, p.vel[3 * i + a]);
        for (int a = 0; a < 3; ++a) put(out, p.force[3 * i + a]);
    }
    if (type == kPlbTypeCapsule) {
        put(out, p.model == BIB_MODEL_CAPSULE_SKALAK ? kShearSkalak : kShearNeoHookean);
        for (int k : kCapsulePack) put(out, p.prm[k]);
    } else {
        for (int k : kRbcPack) put(out, p.prm[k]);
    }
    return true;
}

bool plb_unpack(const char*& it, const char* end, const std::vector<int>& shape_nv, PlbParticle& p,
                std::string& err) {
    int64_t type = -1;
    bool vox = true;
    if (!get(it, end, type) || !get(it, end, p.shape) || !get(it, end, p.id) || !get(it, end, vox)) {
        err = "truncated particle header";
        return false;
    }
    p.voxelize = vox;
    if (type != kPlbTypeCapsule && type != kPlbTypeRbc) {
        err = "unknown particle type " + std::to_string(type);
        return false;
    }
    if (p.shape < 0 || p.shape >= (int64_t)shape_nv.size()) {
        err = "unknown shape id " + std::to_string(p.shape);
        return false;
    }
    const size_t nv = (size_t)shape_nv[p.shape];
    p.pos.resize(3 * nv);
    p.vel.resize(3 * nv);
    p.force.resize(3 * nv);
    for (size_t i = 0; i < nv; ++i) {
        bool ok = true;
        for (int a = 0; a < 3; ++a) ok = ok && get(it, end, p.pos[3 * i + a]);
        for (int a = 0; a < 3; ++a) ok = ok && get(it, end, p.vel[3 * i + a]);
        for (int a = 0; a < 3; ++a) ok = ok && get(it, end, p.force[3 * i + a]);
        if (!ok) {
            err = "truncated vertex data";
            return false;
        }
    }
    for (double& v : p.prm) v = 0.0;
    if (type == kPlbTypeCapsule) {
        int32_t law = -1;
        bool ok = get(it, end, law);
        for (int k : kCapsulePack) ok = ok && get(it, end, p.prm[k]);
        if (!ok || (law != kShearSkalak && law != kShearNeoHookean)) {
            err = "bad capsule parameters";
            return false;
        }
        p.model = law == kShearSkalak ? BIB_MODEL_CAPSULE_SKALAK : BIB_MODEL_CAPSULE_NEOHOOKEAN;
    } else {
        bool ok = true;
        for (int k : kRbcPack) ok = ok && get(it, end, p.prm[k]);
        if (!ok) {
            err = "truncated RBC parameters";
            return false;
        }
        p.model = BIB_MODEL_RBC_WLCPOW;
    }
    return true;
}

std::string vtu_bytes(const double* pos, const double* force, int nv, const int* tri, int nt) {
    const uint64_t sizes[5] = {3ull * nv * sizeof(float), 3ull * nv * sizeof(float), 3ull * nt * sizeof(int32_t),
                               (uint64_t)nt * sizeof(int32_t), (uint64_t)nt * sizeof(int32_t)};
    uint64_t offsets[5];
    offsets[0] = 0;
    for (int i = 1; i < 5; ++i) offsets[i] = offsets[i - 1] + sizeof(uint32_t) + sizes[i - 1];
    std::ostringstream h;
    h << "<?xml version=\"1.0\"?>\n"
      << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt32\" >\n"
      << "  <UnstructuredGrid>\n"
      << "    <Piece NumberOfPoints=\"" << nv << "\" NumberOfCells=\"" << nt << "\" >\n"
      << "      <Points>\n"
      << "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"appended\" offset=\"" << offsets[0]
      << "\" />\n"
      << "      </Points>\n"
      << "      <PointData>\n"
      << "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Name=\"force_tot\" format=\"appended\" offset=\""
      << offsets[1] << "\" />\n"
      << "      </PointData>\n"
      << "      <Cells>\n"
      << "        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"appended\" offset=\"" << offsets[2]
      << "\" />\n"
      << "        <DataArray type=\"Int32\" Name=\"offsets\" format=\"appended\" offset=\"" << offsets[3] << "\" />\n"
      << "        <DataArray type=\"Int32\" Name=\"types\" format=\"appended\" offset=\"" << offsets[4] << "\" />\n"
      << "      </Cells>\n"
      << "    </Piece>\n"
      << "  </UnstructuredGrid>\n"
      << "  <AppendedData encoding=\"raw\">\n"
      << "_";
    std::string out = h.str();
    put(out, (uint32_t)sizes[0]);
    for (int i = 0; i < 3 * nv; ++i) put(out, (float)pos[i]);
    put(out, (uint32_t)sizes[1]);
    for (int i = 0; i < 3 * nv; ++i) put(out, (float)force[i]);
    put(out, (uint32_t)sizes[2]);
    for (int i = 0; i < 3 * nt; ++i) put(out, (int32_t)tri[i]);
    put(out, (uint32_t)sizes[3]);
    for (int i = 0; i < nt; ++i) put(out, (int32_t)(3 * (i + 1)));
    put(out, (uint32_t)sizes[4]);
    for (int i = 0; i < nt; ++i) put(out, (int32_t)5);  // VTK_TRIANGLE
    out += "\n  </AppendedData>\n</VTKFile>\n";
    return out;
}

std::string lightweight_line(const std::string& tag, int64_t id, const double* pos, int nv, const double* com,
                             double volume) {
    // DeformableParticle3D::compute_tensor_of_gyration (DeformableParticle3D.hh:111-125)
    double g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int v = 0; v < nv; ++v)
        for (int i = 0; i < 3; ++i)
            for (int j = i; j < 3; ++j) g[i][j] += (pos[3 * v + i] - com[i]) * (pos[3 * v + j] - com[j]);
    std::ostringstream o;
    o << tag << ":" << id;
    for (int i = 0; i < 3; ++i) o << ":" << com[i];
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) o << ":" << g[i][j] / nv;
    o << ":" << volume;
    return o.str();
}

std::string plb_lattice_xml(const std::string& dat_file, int nx, int ny, int nz, bool vof, int64_t bytes) {
    // XMLwriter::print layout: four spaces per level, "<tag> value </tag>"
    std::ostringstream o;
    const std::string box = "0 " + std::to_string(nx - 1) + " 0 " + std::to_string(ny - 1) + " 0 " + std::to_string(nz - 1);
    o << "<?xml version=\"1.0\" ?>\n"
      << "<Block3D>\n"
      << "    <General>\n"
      << "        <Family> BlockLattice3D </Family>\n"
      << "        <Datatype> double </Datatype>\n"
      << "        <Descriptor> ForcedPhaseD3Q19 </Descriptor>\n"
      << "        <cellDim> 23 </cellDim>\n"
      << "        <dynamicContent> False </dynamicContent>\n"
      << "        <globalId> 0 </globalId>\n"
      << "    </General>\n"
      << "    <Structure>\n"
      << "        <BoundingBox> " << box << " </BoundingBox>\n"
      << "        <EnvelopeWidth> 1 </EnvelopeWidth>\n"
      << "        <GridLevel> 0 </GridLevel>\n"
      << "        <NumComponents> 1 </NumComponents>\n"
      << "    </Structure>\n"
      << "    <Data>\n"
      << "        <File> " << dat_file << " </File>\n"
      << "        <Component> " << box << " </Component>\n"
      << "        <Offsets> " << bytes << " </Offsets>\n";
    if (vof)  // the registered name of GuoExternalForceVOFDynamics and its id in the reference's programs
        o << "        <DynamicsDict>\n"
          << "            <Guo_VOF_dynamics> 3 </Guo_VOF_dynamics>\n"
          << "        </DynamicsDict>\n";
    o << "    </Data>\n"
      << "</Block3D>\n";
    return o.str();
}

namespace {

// text of every leaf element <tag ...> text </tag> of an XML document, in order
std::vector<std::string> xml_leaves(const std::string& xml, const std::string& tag) {
    std::vector<std::string> out;
    const std::string open = "<" + tag, close = "</" + tag + ">";
    size_t at = 0;
    while ((at = xml.find(open, at)) != std::string::npos) {
        const size_t after = at + open.size();
        if (after >= xml.size() || (xml[after] != '>' && xml[after] != ' ' && xml[after] != '\t')) {
            at = after;
            continue;
        }
        const size_t gt = xml.find('>', after);
        if (gt == std::string::npos) break;
        const size_t end = xml.find(close, gt);
        if (end == std::string::npos) break;
        out.push_back(xml.substr(gt + 1, end - gt - 1));
        at = end + close.size();
    }
    return out;
}

std::string trim(const std::string& s) {
    const size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

bool ints(const std::string& s, std::vector<int64_t>& v) {
    std::istringstream in(s);
    v.clear();
    long long x;
    while (in >> x) v.push_back(x);
    return in.eof();
}

bool one(const std::string& xml, const std::string& tag, std::string& v) {
    std::vector<std::string> l = xml_leaves(xml, tag);
    if (l.size() != 1) return false;
    v = trim(l[0]);
    return true;
}

}  // namespace

bool plb_lattice_parse(const std::string& xml, PlbLatticeSpec& s, std::string& err) {
    std::string v;
    std::vector<int64_t> iv;
    if (!one(xml, "cellDim", v) || !ints(v, iv) || iv.size() != 1) return err = "no cellDim", false;
    s.cell_dim = (int)iv[0];
    if (!one(xml, "dynamicContent", v)) return err = "no dynamicContent", false;
    s.dynamic = !(v == "False" || v == "false" || v == "0");
    if (!one(xml, "Datatype", v)) return err = "no Datatype", false;
    s.datatype = v;
    if (!one(xml, "BoundingBox", v) || !ints(v, iv) || iv.size() != 6) return err = "no BoundingBox", false;
    for (int k = 0; k < 6; ++k) s.box[k] = iv[k];
    if (!one(xml, "NumComponents", v) || !ints(v, iv) || iv.size() != 1) return err = "no NumComponents", false;
    const int64_t ncomp = iv[0];
    if (!one(xml, "Offsets", v) || !ints(v, s.offsets)) return err = "no Offsets", false;
    if (!one(xml, "File", v) || v.empty()) return err = "no File", false;
    s.file = v;
    s.ordering.clear();
    one(xml, "IndexOrdering", s.ordering);
    s.comps.clear();
    for (const std::string& c : xml_leaves(xml, "Component")) {
        if (!ints(trim(c), iv) || iv.size() != 6) return err = "malformed Component", false;
        std::array<int64_t, 6> b;
        for (int k = 0; k < 6; ++k) b[k] = iv[k];
        s.comps.push_back(b);
    }
    if ((int64_t)s.comps.size() != ncomp || (int64_t)s.offsets.size() != ncomp)
        return err = "component and offset counts differ from NumComponents", false;
    return true;
}

bool mkdir_p(const std::string& dir) {
    // io::mkdir (src/fsi/IO.hh): every prefix ending at a '/' and the whole path
    std::string cur;
    for (size_t i = 0; i <= dir.size(); ++i) {
        if (i == dir.size() || dir[i] == '/') {
            if (!cur.empty() && cur != "/") {
                struct stat st;
                if (stat(cur.c_str(), &st) != 0) {
                    if (::mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) return false;
                } else if (!S_ISDIR(st.st_mode)) {
                    return false;
                }
            }
        }
        if (i < dir.size()) cur += dir[i];
    }
    return true;
}

}  // namespace bib
