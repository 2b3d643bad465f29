// noalloc.cu -- J/K build that needs no device allocation by the caller.
//
// sq_jk's FP32 launches need an nbf x nbf FP32 copy of the density as scratch,
// which the caller normally allocates and passes in.  Some callers cannot do
// that: a host framework that has already claimed all device memory for its
// own pool (and forbids other cudaMalloc calls), code running on a stream
// whose capture mode does not allow allocations, and tight SCF loops where the
// implicit device synchronisation of cudaMalloc/cudaFree is not acceptable.
// sq_jk_noalloc serves them: the scratch is a fixed-size array in this
// library's own device memory, reserved when the library is loaded.
//
// Limits and behaviour:
//   * the density handed to the FP32 launches holds at most
//     SQ_NOALLOC_MAX_ELEMS (1024 x 1024) elements: nbf <= 1024 for one
//     molecule, and a packed batch basis (mat_base != NULL) must have
//     mat_total = sum_i n_i^2 <= 1024 x 1024 whatever its nbf (nbf of a batch
//     is only its largest molecule).  The array is 4 MiB on every GPU that
//     loads the library, held until the process exits; larger inputs are
//     rejected with SQ_ERR_ARG before anything is launched;
//   * every call (whatever its precision) first makes sure the array's device
//     address is known for the current device: the first call on a device
//     looks it up (cudaGetSymbolAddress, with that device current) and caches
//     it, so make that first call before any stream capture;
//   * every call shares the one array: calls that overlap on the GPU (two
//     streams, or two host threads) race on it and must be serialised by the
//     caller.  The array keeps the last call's FP32 density; nothing in it has
//     to start at zero because each FP32 call overwrites its first mat_total
//     elements before reading them;
//   * no cudaMalloc, cudaFree or allocating library routine is called.
#include <mutex>

#include "capi_internal.cuh"
#include "sq_common.cuh"

namespace {

constexpr int kMaxDevices = 64;

// File-scope scratch: the FP32 copy of the density matrix.
static __device__ __align__(256) float g_density32_scratch[SQ_NOALLOC_MAX_ELEMS];

std::mutex g_scratch_mutex;
float *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once per
// device; the host-side symbol itself is not a device address).
int scratch_address(float **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sq::set_error(SQ_ERR_CUDA, "sq_jk_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return sq::set_error(SQ_ERR_ARG, "sq_jk_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_density32_scratch);
        if (e != cudaSuccess || p == nullptr)
            return sq::set_error(SQ_ERR_CUDA, "sq_jk_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                                 cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<float *>(p);
    }
    *out = g_scratch_addr[dev];
    return SQ_OK;
}

}  // namespace

extern "C" int sq_jk_noalloc(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                             const sq_quartets *quartets, const double *table64, const float *table32, const double *D,
                             double *Jacc, double *Kacc, int precision, void *stream) {
    if (!basis) return sq::set_error(SQ_ERR_ARG, "sq_jk_noalloc: basis is NULL");
    if (basis->nbf < 0 || basis->nbf > SQ_NOALLOC_MAX_NBF)
        return sq::set_error(SQ_ERR_ARG,
                             "sq_jk_noalloc: nbf = %d exceeds the static scratch limit of %d basis functions "
                             "(use sq_jk with caller-allocated scratch)",
                             basis->nbf, SQ_NOALLOC_MAX_NBF);
    // the FP32 density covers mat_total elements: n^2 for one molecule, the
    // packed length sum_i n_i^2 for a batch (whose nbf is its largest molecule)
    const long long mt = sq::mat_total(*basis);
    if (mt < 0 || mt > (long long)SQ_NOALLOC_MAX_ELEMS)
        return sq::set_error(SQ_ERR_ARG,
                             "sq_jk_noalloc: the density holds %lld elements, which exceeds the static scratch "
                             "limit of %lld elements (use sq_jk with caller-allocated scratch)",
                             mt, (long long)SQ_NOALLOC_MAX_ELEMS);
    // resolved on every call, FP64 ones included, so that the first call on a
    // device (whatever its precision) is the one that looks the address up
    float *d32 = nullptr;
    const int rc = scratch_address(&d32);
    if (rc != SQ_OK) return rc;
    // serial launches on the caller's stream: the library's stream pool would
    // create streams and events on its first use
    return sq::jk_serial(basis, pairs, slots, quartets, table64, table32, D, precision == SQ_FP64 ? nullptr : d32, Jacc,
                         Kacc, precision, stream);
}
