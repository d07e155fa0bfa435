// pg_bin_particles_noalloc: cell binning with library-owned scratch.
//
// Some callers cannot allocate device memory when they bin: a host code that
// hands the library a fixed memory budget at start-up and forbids any allocation
// afterwards, or a caller that must not pay for (or risk failing) a device
// allocation in the middle of its time loop.  pg_bin_particles needs a caller-made
// workspace; this variant instead uses a fixed scratch array that lives in the
// library's own device image, so the caller passes only inputs and outputs.
//
// The scratch is a file-scope __device__ array of kNoAllocBytes bytes (enough for
// PG_NOALLOC_MAX_PARTICLES particles in a grid of at most PG_NOALLOC_MAX_CELLS
// cells).  Every GPU that loads the library holds this array until the process
// exits.  Host code cannot use the array's name as a device pointer (on the host
// it names a host-side shadow), so its device address is looked up once per device
// with cudaGetSymbolAddress and cached.
#include "common.cuh"

#include <atomic>

namespace pg {

int bin_particles(const pg_box *box, pg_particles *p, pg_cells *cells, pg_workspace ws, pg_status *status,
                  cudaStream_t st, int32_t **perm_out);
int64_t bin_workspace_bytes(int32_t n, int32_t ncells);
bool grid_ok(const pg_cells *cells);

// Size of the binning workspace for the limits above, following the layout of
// bin_particles' workspace: cell counts, starts and cursors for ncells + 2 entries,
// the scan's block sums, the permutation (4 B per particle) and the gather staging
// area (88 B per particle: every per-particle array at once), each rounded up to 256
// bytes.  The call below checks bin_workspace_bytes against this size, so a change
// of the layout cannot leave the array too small.
constexpr size_t round256(size_t x) { return (x + 255) & ~(size_t) 255; }
constexpr size_t noalloc_bytes(size_t n, size_t ncells) {
    return round256((ncells + 2) * 4) + round256((ncells + 3) * 4) + round256((ncells + 2) * 4) +
           round256(((ncells + 2 + 1023) / 1024 + 1) * 4) + round256(n * 4) + round256(n * 88);
}
constexpr size_t kNoAllocBytes = noalloc_bytes(PG_NOALLOC_MAX_PARTICLES, PG_NOALLOC_MAX_CELLS);

static __device__ __align__(256) unsigned char g_bin_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
static std::atomic<void *> g_scratch_addr[kMaxDevices];

// Device address of g_bin_scratch on the current device (looked up on first use).
static int scratch_address(void **out) {
    int dev = -1;
    if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) { return PG_ERR_CUDA; }
    void *ptr = g_scratch_addr[dev].load(std::memory_order_acquire);
    if(ptr == nullptr) {
        if(cudaGetSymbolAddress(&ptr, g_bin_scratch) != cudaSuccess || ptr == nullptr) { return PG_ERR_CUDA; }
        g_scratch_addr[dev].store(ptr, std::memory_order_release);
    }
    *out = ptr;
    return PG_OK;
}

}  // namespace pg

extern "C" int pg_bin_particles_noalloc(const pg_box *box, pg_particles *p, pg_cells *cells, pg_status *status,
                                        void *stream) {
    if(box == nullptr || p == nullptr || cells == nullptr || status == nullptr) { return PG_ERR_ARGUMENT; }
    if(p->n < 0 || !pg::grid_ok(cells)) { return PG_ERR_ARGUMENT; }
    if(p->n > PG_NOALLOC_MAX_PARTICLES || cells->ncells > PG_NOALLOC_MAX_CELLS) { return PG_ERR_LIMIT; }
    const int64_t need = pg::bin_workspace_bytes(p->n, cells->ncells);
    if(need < 0 || (size_t) need > pg::kNoAllocBytes) { return PG_ERR_LIMIT; }
    void *scratch = nullptr;
    const int rc = pg::scratch_address(&scratch);
    if(rc != PG_OK) { return rc; }
    // The cell counters in the scratch are cleared by bin_particles itself (a memset
    // on the stream before counting); nothing else is read before it is written.
    pg_workspace ws;
    ws.ptr = scratch;
    ws.bytes = (int64_t) pg::kNoAllocBytes;
    return pg::bin_particles(box, p, cells, ws, status, reinterpret_cast<cudaStream_t>(stream), nullptr);
}
