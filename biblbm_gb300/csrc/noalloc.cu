// Deterministic force spreading that allocates no device memory.
//
// Some callers cannot let a library allocate device memory.  A host application that has
// handed the GPU's memory to its own pool allocator (a co-processor driver that reserves
// HBM for its lattices at start-up, or a framework whose caching allocator holds the free
// memory) would see a cudaMalloc from the library fail or fragment its pool; a
// time-critical stepping loop cannot afford the device-wide synchronisation that
// cudaMalloc / cudaFree imply.  The ordinary deterministic spreading of a lattice keeps
// its sort buffers in device memory allocated when the particles are uploaded; this file
// gives the same computation a fixed scratch area instead: one file-scope device array,
// sized for BIB_SPREAD_NOALLOC_MAX_ENTRIES (cell, entry) pairs plus the radix sort's
// temporary storage.
//
// Layout of the array: keys[2] and ids[2] (BIB_SPREAD_NOALLOC_MAX_ENTRIES 32-bit words
// each), then the sort's temporary storage.  Nothing in it has to start at zero: every
// call writes the keys and ids it sorts, and the sort initialises its own temporaries.
// All calls share the one array, so calls that overlap in time on one device race on it.
//
// The host needs the array's device address to pass it to the kernels: the array's name in
// host code is a host-side stand-in, not a device address.  bib_create resolves it with
// cudaGetSymbolAddress while the context's device is current (the set-up step) and keeps it in
// the context; a context created after a cudaDeviceReset therefore holds the address in the
// new device context, and the entry point itself makes no runtime query that a stream capture
// would have to record.
#include <string>

#include "bib_internal.h"

namespace bib {

constexpr size_t kNoallocEntries = (size_t)BIB_SPREAD_NOALLOC_MAX_ENTRIES;
constexpr size_t kNoallocSortTemp = (size_t)BIB_SPREAD_NOALLOC_SCRATCH_BYTES - 4 * sizeof(uint32_t) * kNoallocEntries;
static_assert(BIB_SPREAD_NOALLOC_SCRATCH_BYTES > 4 * sizeof(uint32_t) * BIB_SPREAD_NOALLOC_MAX_ENTRIES,
              "scratch must hold the keys, the ids and the sort's temporary storage");

static __device__ __align__(256) unsigned char g_spread_scratch[BIB_SPREAD_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array on the current device (the set-up step, run by bib_create).
bib_status spread_scratch_address(void** out, std::string& msg) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_spread_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        msg = std::string("cudaGetSymbolAddress of the spreading scratch failed: ") + cudaGetErrorString(e);
        return BIB_ECUDA;
    }
    *out = p;
    return BIB_OK;
}

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

bib_status spread_noalloc(const Lattice& L, int device, void* scratch, cudaStream_t s, const double* pos,
                          const double* force, int64_t nvert, void* field, std::string& msg) {
    if (nvert < 0) {
        msg = "negative vertex count";
        return BIB_EINVAL;
    }
    const int64_t sup = L.ib.dirac == BIB_DIRAC_PESKIN ? 4 : 3;
    const int64_t ne = nvert * sup * sup * sup;
    if (ne > (int64_t)kNoallocEntries) {
        msg = "nvert x support^3 = " + std::to_string(ne) + " exceeds BIB_SPREAD_NOALLOC_MAX_ENTRIES = " +
              std::to_string(kNoallocEntries) + " (at most " + std::to_string(kNoallocEntries / (sup * sup * sup)) +
              " vertices with this kernel)";
        return BIB_EINVAL;
    }
    if (L.ib.has_pipe) {
        msg = "the spreading scratch path does not blend kernels near a pipe boundary";
        return BIB_EUNSUPPORTED;
    }
    if (L.d.n >= (int64_t)0xffffffff) {
        msg = "lattice too large for 32-bit cell keys";
        return BIB_EUNSUPPORTED;
    }
    if (nvert == 0) return BIB_OK;
    if (!pos || !force || !field) {
        msg = "null device pointer";
        return BIB_EINVAL;
    }
    const int end_bit = spread_key_bits(L.d.n);
    const size_t temp = spread_sort_temp_bytes_pingpong(ne, end_bit);
    if (temp > kNoallocSortTemp) {
        msg = "radix sort needs " + std::to_string(temp) + " bytes of temporary storage, the scratch holds " +
              std::to_string(kNoallocSortTemp);
        return BIB_EUNSUPPORTED;
    }
    if (!scratch) {
        msg = "the context holds no address of the spreading scratch";
        return BIB_ECUDA;
    }
    DeviceGuard guard(device);
    uint32_t* words = static_cast<uint32_t*>(scratch);
    uint32_t* keys0 = words;
    uint32_t* keys1 = words + kNoallocEntries;
    uint32_t* ids0 = words + 2 * kNoallocEntries;
    uint32_t* ids1 = words + 3 * kNoallocEntries;
    void* sort_temp = words + 4 * kNoallocEntries;
    // the caller's field is dense: component c of cell k at field[c * n + k]
    LatticeDesc d = L.d;
    d.stride = d.n;
    const cudaError_t e = launch_spread_sorted(d, L.ib, L.storage == BIB_STORAGE_F64, (int)nvert, pos, force, field,
                                               keys0, keys1, ids0, ids1, sort_temp, kNoallocSortTemp, s);
    if (e != cudaSuccess) {
        msg = std::string("spreading launch failed: ") + cudaGetErrorString(e);
        return BIB_ECUDA;
    }
    return BIB_OK;
}

}  // namespace bib
