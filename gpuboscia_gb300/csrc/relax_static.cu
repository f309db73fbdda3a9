// relax_static.cu -- gbx_relax_batch_static: the batched relaxation with its
// scratch memory inside the library instead of in a caller-provided buffer.
//
// Who needs it: callers that cannot allocate device memory when they relax a
// batch -- a host language bound over the C ABI without access to a CUDA
// allocator, a process whose device memory is owned by another runtime's pool,
// or a latency-critical loop where an allocation (and its implicit
// synchronisation) is not allowed. They still own the node buffers (inputs and
// outputs); only the scratch moves here.
//
// The scratch is one file-scope __device__ array of GBX_STATIC_SCRATCH_BYTES.
// Every GPU that loads this library keeps it until the process exits. Its
// device address is looked up with cudaGetSymbolAddress on the first call on
// each device (with that device current); that first call should come before
// any stream capture. All calls share the array and it keeps the last call's
// contents: the relaxation writes every scratch word before reading it, so
// nothing has to start at zero. Calls that overlap on the GPU (other streams,
// other host threads) race on the array: issue them on one stream.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "relax.cuh"

namespace {

static __device__ __align__(256) unsigned char g_static_scratch[GBX_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (looked up once).
int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        gbx::set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return GBX_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        gbx::set_last_error("device index beyond the static scratch table");
        return GBX_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            gbx::set_last_error(std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
            return GBX_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GBX_OK;
}

}  // namespace

extern "C" int gbx_relax_batch_static(const gbx_objective* obj, const gbx_lmo* lmo,
                                      const gbx_algorithm* alg, const gbx_node_batch* batch,
                                      void* stream) {
    if (!batch) {
        gbx::set_last_error("batch: null descriptor");
        return GBX_ERR_INVALID;
    }
    if (batch->n_nodes < 0 || batch->max_iters < 0) {
        gbx::set_last_error("batch: n_nodes and max_iters must be non-negative");
        return GBX_ERR_INVALID;
    }
    const size_t need = gbx_relax_workspace_bytes(obj, lmo, alg, batch->n_nodes);
    if (need == 0) return GBX_ERR_INVALID;  // bad descriptors: the sizing call set the message
    if (need > GBX_STATIC_SCRATCH_BYTES) {
        gbx::set_last_error("batch needs " + std::to_string(need) + " bytes of scratch; the static scratch holds " +
                            std::to_string((size_t)GBX_STATIC_SCRATCH_BYTES) +
                            " (split the batch or use gbx_relax_batch with a workspace)");
        return GBX_ERR_WORKSPACE;
    }
    void* scratch = nullptr;
    const int rc = scratch_address(&scratch);
    if (rc != GBX_OK) return rc;
    return gbx_relax_batch(obj, lmo, alg, batch, scratch, GBX_STATIC_SCRATCH_BYTES, stream);
}
