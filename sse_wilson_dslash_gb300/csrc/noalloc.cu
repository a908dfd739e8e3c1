// The packed-layout Dslash without any allocation (gbds_dslash_packed_noalloc_f32
// in gbdslash.h).  It runs the same pack -> Dslash -> unpack kernels as the
// host-pointer path, with the structure-of-arrays copies placed in a
// file-scope device array instead of memory from cudaMalloc.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "gbds_internal.h"

namespace {

// Largest lattice: 32768 sites, i.e. a 16384-site checkerboard (a multiple of
// 64, so stride = Vh).  FP32, 18-real links, 4D:
//   gauge 2 * 4 * 72 B * 16384 = 9 MiB, two spinor checkerboards 2 * 96 B * 16384 = 3 MiB.
static_assert(GBDS_NOALLOC_SCRATCH_BYTES == 2 * 4 * 72 * (GBDS_NOALLOC_MAX_SITES / 2) +
                                               2 * 96 * (GBDS_NOALLOC_MAX_SITES / 2),
              "scratch size must match the site limit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[GBDS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  In host code
// the array's name only stands in for the symbol; the address must come from
// the runtime, once per device, with that device current.
int scratch_address(void **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return gbds::cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return gbds::set_error(GBDS_ERROR_UNSUPPORTED, "device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return gbds::cuda_error(e, "cudaGetSymbolAddress(no-allocation scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GBDS_SUCCESS;
}

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" int gbds_dslash_packed_noalloc_f32(const int dims[4], int nd, const float *u_packed,
                                              const float *psi_packed, float *res_packed, int isign, int cb,
                                              void *stream) {
    gbds::Geom g;
    int rc = gbds::make_geom(dims, nd, &g);
    if (rc != GBDS_SUCCESS) return rc;
    if (g.V > GBDS_NOALLOC_MAX_SITES) {
        char b[200];
        snprintf(b, sizeof b,
                 "gbds_dslash_packed_noalloc_f32: lattice of %d sites exceeds the no-allocation limit of %d sites "
                 "(%d bytes of static scratch); use the gbds_op_* path with caller buffers",
                 g.V, GBDS_NOALLOC_MAX_SITES, GBDS_NOALLOC_SCRATCH_BYTES);
        return gbds::set_error(GBDS_ERROR_INVALID_VALUE, b);
    }
    if (isign != 1 && isign != -1) return GBDS_SUCCESS;
    if (cb != 0 && cb != 1) return gbds::set_error(GBDS_ERROR_INVALID_VALUE, "cb must be 0 or 1");
    if (!u_packed || !psi_packed || !res_packed) return gbds::set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    if (!aligned16(u_packed) || !aligned16(psi_packed) || !aligned16(res_packed))
        return gbds::set_error(GBDS_ERROR_INVALID_VALUE, "fields must be 16-byte aligned");

    const size_t gauge_b = align256(gbds::gauge_bytes(g, 32, 18));
    const size_t spin_b = align256(gbds::spinor_bytes(g, 32));
    if (gauge_b + 2 * spin_b > (size_t)GBDS_NOALLOC_SCRATCH_BYTES)
        return gbds::set_error(GBDS_ERROR_INVALID_VALUE, "no-allocation scratch too small for this lattice");

    void *base = nullptr;
    rc = scratch_address(&base);
    if (rc != GBDS_SUCCESS) return rc;
    char *s = static_cast<char *>(base);
    void *gauge = s, *src = s + gauge_b, *dst = s + gauge_b + spin_b;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = gbds::launch_pack_gauge(g, 32, 18, u_packed, nullptr, gauge, st);
    if (e == cudaSuccess) e = gbds::launch_pack_spinor(g, 32, psi_packed, nullptr, 0, cb, src, st);
    if (e == cudaSuccess) e = gbds::launch_dslash_f32(g, 18, gauge, src, dst, isign, cb, 0, 0, st);
    if (e == cudaSuccess) e = gbds::launch_unpack_spinor(g, 32, dst, nullptr, 0, 1 - cb, res_packed, st);
    return e == cudaSuccess ? GBDS_SUCCESS : gbds::cuda_error(e, "gbds_dslash_packed_noalloc_f32");
}
