// Extended C ABI (gbdslash.h): operator handles on device pointers, status
// codes, and the implementation of the reference's host-pointer entry points
// (init / free / apply / pack) behind precision-suffixed names.
#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbds_internal.h"

namespace gbds {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

int set_error(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int cuda_error(cudaError_t e, const char *where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return set_error(e == cudaErrorMemoryAllocation ? GBDS_ERROR_OUT_OF_MEMORY : GBDS_ERROR_CUDA, m);
}

void count_launch(int n) { g_launches += n; }

int make_geom(const int dims[4], int nd, Geom *g) {
    if (!dims) return set_error(GBDS_ERROR_INVALID_VALUE, "dims is NULL");
    if (nd != 3 && nd != 4) return set_error(GBDS_ERROR_INVALID_VALUE, "nd must be 3 or 4");
    long long V = 1;
    for (int mu = 0; mu < 4; mu++) {
        if (dims[mu] <= 0) return set_error(GBDS_ERROR_INVALID_VALUE, "lattice extents must be positive");
        if (mu < nd && dims[mu] % 2 != 0) {
            char b[160];
            snprintf(b, sizeof b, "lattice extent %d in direction %d is odd; the %dD operator needs even dims%s", dims[mu],
                     mu, nd, nd == 3 ? " 0..2" : "");
            return set_error(GBDS_ERROR_INVALID_VALUE, b);
        }
        V *= dims[mu];
    }
    if (V > (1LL << 30)) return set_error(GBDS_ERROR_UNSUPPORTED, "lattice volume above 2^30 sites");
    for (int mu = 0; mu < 4; mu++) g->L[mu] = dims[mu];
    g->nd = nd;
    g->Lxh = dims[0] / 2;
    g->V = (int)V;
    g->Vh = (int)(V / 2);
    g->stride = (g->Vh + 63) / 64 * 64;
    g->zblock = 0;
    return GBDS_SUCCESS;
}

// The neighbour reuse of a multi-RHS launch in the natural site order spans
// 2 Lz (z, t) planes of traffic (a source plane is read by the output planes
// at t - 1 and t + 1); beyond about kGenReuseBytes it falls out of the 129 MB
// L2 and source spinors are read from DRAM more than once (32^3x64, 16 rhs
// in FP32 pairs: DRAM reads 2.2x the compulsory bytes).  The z slab keeps the
// span at 2 B planes; its z faces cost 2 / B extra source reads, so B is the
// largest divisor of Lz that fits.  Measured on GB300: 32^3x64 and 40^4 with
// 16 rhs 8-11 % faster in slabs, 24^3x48 with 16 rhs (a 48 MB span) and
// BF16 with 32 rhs faster in the natural order.
constexpr double kGenReuseBytes = 64e6;

int gen_zblock(const Geom &g, int nrhs, int fmt, int recon) {
    if (g.nd != 4) return 0;
    const double site = (double)nrhs * 2 * gen_spinor_bytes(fmt) + 8.0 * recon * 4;  // source, target, 8 links
    const double plane = site * g.Lxh * g.L[1];
    if (2.0 * g.L[2] * plane <= kGenReuseBytes) return 0;
    int best = 1;
    for (int b = 2; b < g.L[2] && b < 32768; b++)  // Geom holds it in 16 bits
        if (g.L[2] % b == 0 && 2.0 * b * plane <= kGenReuseBytes) best = b;
    return best;
}

// Coordinates of internal site i (= p*Vh + h) in the operator's canonical order.
static void internal_coords(const Geom &g, int i, int c[4]) {
    const int p = i / g.Vh;
    int r = i % g.Vh;
    if (g.nd == 4) {
        const int xh = r % g.Lxh; r /= g.Lxh;
        c[1] = r % g.L[1]; r /= g.L[1];
        c[2] = r % g.L[2];
        c[3] = r / g.L[2];
        c[0] = 2 * xh + ((p + c[1] + c[2] + c[3]) & 1);
    } else {
        c[3] = r % g.L[3]; r /= g.L[3];
        const int xh = r % g.Lxh; r /= g.Lxh;
        c[1] = r % g.L[1];
        c[2] = r / g.L[1];
        c[0] = 2 * xh + ((p + c[1] + c[2]) & 1);
    }
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace gbds

using namespace gbds;

// ---------------------------------------------------------------------------
// Operator handle
// ---------------------------------------------------------------------------

extern "C" const char *gbds_get_last_error(void) { return g_last_error.c_str(); }

extern "C" long long gbds_kernel_launch_count(void) { return g_launches.load(); }

extern "C" int gbds_op_create(gbds_op *op, const int dims[4], int nd, int prec, int recon) {
    return gbds_op_create_ex(op, dims, nd, prec, recon, 1, GBDS_SPINOR_NATIVE);
}

extern "C" int gbds_op_create_ex(gbds_op *op, const int dims[4], int nd, int prec, int recon, int nrhs, int format) {
    if (!op) return set_error(GBDS_ERROR_INVALID_VALUE, "op is NULL");
    *op = nullptr;
    if (prec != 32 && prec != 64) return set_error(GBDS_ERROR_INVALID_VALUE, "prec must be 32 or 64");
    if (recon != 18 && recon != 12) return set_error(GBDS_ERROR_INVALID_VALUE, "recon must be 18 or 12");
    if (nrhs < 1 || nrhs > 32) return set_error(GBDS_ERROR_INVALID_VALUE, "nrhs must be in [1, 32]");
    if (format != GBDS_SPINOR_NATIVE && format != GBDS_SPINOR_BF16 && format != GBDS_SPINOR_F16_NORM &&
        format != GBDS_SPINOR_F32_PAIRS && format != GBDS_SPINOR_DOUBLE_FLOAT)
        return set_error(GBDS_ERROR_INVALID_VALUE, "unknown spinor format");
    if (format == GBDS_SPINOR_DOUBLE_FLOAT && (prec != 64 || nrhs != 1))
        return set_error(GBDS_ERROR_UNSUPPORTED, "the double-float format needs prec 64 and one right-hand side");
    if ((nrhs > 1 || (format != GBDS_SPINOR_NATIVE && format != GBDS_SPINOR_DOUBLE_FLOAT)) && (prec != 32 || nd != 4))
        return set_error(GBDS_ERROR_UNSUPPORTED,
                         "several right-hand sides and the non-native spinor formats need prec 32 and nd 4");
    Geom g;
    int rc = make_geom(dims, nd, &g);
    if (rc != GBDS_SUCCESS) return rc;
    gbds_op o = new (std::nothrow) gbds_op_s;
    if (!o) return set_error(GBDS_ERROR_OUT_OF_MEMORY, "host allocation failed");
    o->g = g;
    o->prec = prec;
    o->recon = recon;
    // Defaults from a sweep on GB300 at 32^3x64 and 24^3x48 (gbds_op_autotune
    // refines them per lattice): FP32 recon 18 runs best with registers capped
    // for 6 blocks of 128 threads per SM, FP32 recon 12 with 64-thread blocks,
    // FP64 (FP64-issue bound) is insensitive.
    o->block = (prec == 32 && recon == 12) ? 64 : 128;
    o->nrhs = nrhs;
    o->format = format;
    // Single rhs: the register-cap variant (see above).  Several rhs or
    // another format: variant 0 = the plain multi-RHS kernel, 1 = its packed
    // FP32x2 colour multiply, 2 = the whole hop packed, 3 = the same with two
    // rhs a thread, 4 = 3 with cp.async prefetching (16-bit storage);
    // autotune chooses per shape.
    const bool gen = nrhs > 1 || (format != GBDS_SPINOR_NATIVE && format != GBDS_SPINOR_DOUBLE_FLOAT);
    // from 16 rhs on: for 16-bit storage the fully packed kernel with two rhs
    // a thread and cp.async prefetching (variant 4), for both FP32 layouts
    // the same without prefetching (3)
    const int gen_variant =
        nrhs >= 16 ? (format == GBDS_SPINOR_BF16 || format == GBDS_SPINOR_F16_NORM ? 4 : 3)
                   : (nrhs == 8 && format == GBDS_SPINOR_F16_NORM ? 2 : 0);  // 24^3x48, 8 rhs: 0.226 -> 0.182 ms
    o->variant = gen ? gen_variant : ((prec == 32 && recon == 18) ? 1 : 0);
    if (gen) o->g.zblock = gen_zblock(g, nrhs, format, recon);
    o->tensor_cores = 0;
    o->d_err = nullptr;
    o->d_site_table = nullptr;
    *op = o;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_destroy(gbds_op op) {
    if (!op) return GBDS_SUCCESS;
    if (op->d_site_table) cudaFree(op->d_site_table);
    if (op->d_err) cudaFree(op->d_err);
    delete op;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_set_layout(gbds_op op, const int *site_table, int n) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (op->d_site_table) {
        cudaFree(op->d_site_table);
        op->d_site_table = nullptr;
    }
    if (!site_table) return GBDS_SUCCESS;
    const Geom &g = op->g;
    if (n != g.V) return set_error(GBDS_ERROR_INVALID_VALUE, "site_table must have V entries");
    std::vector<char> seen(g.V, 0);
    bool identity = true;
    for (int i = 0; i < g.V; i++) {
        const int c = site_table[i];
        if (c < 0 || c >= g.V || seen[c]) return set_error(GBDS_ERROR_INVALID_VALUE, "site_table is not a permutation of [0, V)");
        seen[c] = 1;
        identity &= (c == i);
    }
    if (identity) return GBDS_SUCCESS;
    cudaError_t e = cudaMalloc(&op->d_site_table, sizeof(int) * (size_t)g.V);
    if (e != cudaSuccess) {
        op->d_site_table = nullptr;
        return cuda_error(e, "cudaMalloc(site_table)");
    }
    e = cudaMemcpy(op->d_site_table, site_table, sizeof(int) * (size_t)g.V, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "cudaMemcpy(site_table)");
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_is_canonical(gbds_op op) { return op && op->d_site_table == nullptr; }

// the multi-RHS / reduced-storage kernels (FP32 arithmetic)
static bool generic(gbds_op op) {
    return op->nrhs > 1 || (op->format != GBDS_SPINOR_NATIVE && op->format != GBDS_SPINOR_DOUBLE_FLOAT);
}
static bool double_float(gbds_op op) { return op->format == GBDS_SPINOR_DOUBLE_FLOAT; }

extern "C" size_t gbds_op_spinor_bytes(gbds_op op) {
    if (!op) return 0;
    if (generic(op)) return (size_t)gen_spinor_bytes(op->format) * op->g.stride * op->nrhs;
    return spinor_bytes(op->g, op->prec);
}

extern "C" int gbds_op_nrhs(gbds_op op) { return op ? op->nrhs : 0; }

extern "C" int gbds_op_set_tensor_cores(gbds_op op, int on) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (on && ((op->format != GBDS_SPINOR_BF16 && op->format != GBDS_SPINOR_F16_NORM) ||
               (op->nrhs != 16 && op->nrhs != 32)))
        return set_error(GBDS_ERROR_UNSUPPORTED, "tensor cores need a 16-bit spinor format and 16 or 32 right-hand sides");
    if (on && !op->d_err) {
        cudaError_t e = cudaMalloc(&op->d_err, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(op->d_err, 0, sizeof(int));
        if (e != cudaSuccess) return cuda_error(e, "gbds_op_set_tensor_cores");
    }
    op->tensor_cores = on ? 1 : 0;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_check(gbds_op op) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (!op->d_err) return GBDS_SUCCESS;
    int v = 0;
    cudaError_t e = cudaMemcpy(&v, op->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "gbds_op_check");
    if (v) {
        cudaMemset(op->d_err, 0, sizeof(int));
        if (v == 2)
            return set_error(GBDS_ERROR_CUDA, "a tensor-core Dslash launch timed out waiting for its MMAs, which "
                                              "had still not completed when its tensor memory was released");
        return set_error(GBDS_ERROR_CUDA, "a tensor-core Dslash launch timed out waiting for its MMAs");
    }
    return GBDS_SUCCESS;
}

extern "C" int gbds_tc_wait_selftest(int polls) {
    if (polls <= 0) return set_error(GBDS_ERROR_INVALID_VALUE, "polls must be positive");
    int *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e != cudaSuccess) return cuda_error(e, "gbds_tc_wait_selftest");
    int flag = -1;
    e = cudaMemset(d, 0xff, sizeof(int));
    if (e == cudaSuccess) e = launch_tc_wait_selftest(polls, d, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(&flag, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_error(e, "gbds_tc_wait_selftest");
    return flag == 2 ? GBDS_SUCCESS : set_error(GBDS_ERROR_CUDA, "the bounded wait did not report its time-out");
}

extern "C" size_t gbds_op_gauge_bytes(gbds_op op) { return op ? gauge_bytes(op->g, op->prec, op->recon) : 0; }

extern "C" int gbds_op_geometry(gbds_op op, int *volume, int *volume_cb, int *stride) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (volume) *volume = op->g.V;
    if (volume_cb) *volume_cb = op->g.Vh;
    if (stride) *stride = op->g.stride;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_set_tuning(gbds_op op, int threads, int variant) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (threads != 0 && (threads < 32 || threads > 256 || threads % 32 != 0))
        return set_error(GBDS_ERROR_INVALID_VALUE, "block must be 0 or a multiple of 32 in [32, 256]");
    if (variant < 0 || variant >= gbds_op_num_variants(op))
        return set_error(GBDS_ERROR_INVALID_VALUE, "variant out of range");
    op->block = threads;
    op->variant = variant;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_set_site_order(gbds_op op, int zblock) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    const int Lz = op->g.L[2];
    if (zblock == -1) {
        op->g.zblock = generic(op) ? gen_zblock(op->g, op->nrhs, op->format, op->recon) : 0;
        return GBDS_SUCCESS;
    }
    if (zblock < 0 || zblock > Lz || (zblock > 0 && Lz % zblock != 0))
        return set_error(GBDS_ERROR_INVALID_VALUE, "zblock must be -1, 0 or a divisor of the z extent");
    if (zblock == Lz) zblock = 0;  // one slab: the natural order
    if (zblock > 32767) return set_error(GBDS_ERROR_UNSUPPORTED, "z slabs of more than 32767 planes");
    if (zblock != 0 && !generic(op))
        return set_error(GBDS_ERROR_UNSUPPORTED, "the site order applies to operators with several right-hand sides "
                                                 "or 16-bit storage");
    op->g.zblock = zblock;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_get_site_order(gbds_op op, int *zblock) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (zblock) *zblock = op->g.zblock;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_num_variants(gbds_op op) {
    if (!op) return 0;
    // 2: the fully packed kernel; 3: the same, two rhs a thread; 4: 3 with
    // cp.async prefetching (16-bit storage)
    if (generic(op)) return 5;
    return double_float(op) ? dslash_variants_df() : dslash_variants(op->prec);
}

namespace {
std::mutex g_tune_mutex;
// (dims, nd, prec, recon, nrhs, format) -> (block, variant, tensor cores,
// z slab of the site order)
std::map<std::array<int, 9>, std::array<int, 4>> g_tune_cache;
}  // namespace

static bool tc_eligible(gbds_op op) {
    return (op->format == GBDS_SPINOR_BF16 || op->format == GBDS_SPINOR_F16_NORM) && (op->nrhs == 16 || op->nrhs == 32);
}

extern "C" int gbds_op_autotune(gbds_op op, const void *gauge, const void *psi, void *res, void *stream) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    // several right-hand sides: the candidates are the plain kernel, its
    // packed FP32x2 form (8, 16, 32 rhs), for 16-bit and FP32-pair storage the
    // fully packed kernel with one and with two rhs a thread, for 16-bit
    // storage the latter with cp.async prefetching and, with 16 or 32 rhs,
    // the tensor-core kernel
    const bool v2ok = op->nrhs == 8 || op->nrhs == 16 || op->nrhs == 32;
    if (generic(op) && !tc_eligible(op) && !v2ok) return GBDS_SUCCESS;
    const std::array<int, 9> key = {op->g.L[0], op->g.L[1], op->g.L[2], op->g.L[3], op->g.nd,
                                    op->prec,   op->recon,  op->nrhs,   op->format};
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            op->block = it->second[0];
            op->variant = it->second[1];
            op->g.zblock = (short)it->second[3];
            return it->second[2] ? gbds_op_set_tensor_cores(op, 1) : gbds_op_set_tensor_cores(op, 0);
        }
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<std::array<int, 3>> cand;
    if (generic(op)) {
        cand = {{op->block, 0, 0}};
        if (v2ok) cand.push_back({op->block, 1, 0});
        if (v2ok) {
            cand.push_back({op->block, 2, 0});
            cand.push_back({op->block, 3, 0});
            if (op->format == GBDS_SPINOR_BF16 || op->format == GBDS_SPINOR_F16_NORM) cand.push_back({op->block, 4, 0});
        }
        if (tc_eligible(op)) cand.push_back({op->block, 0, 1});
    } else {
        cand = {{64, 0, 0}, {128, 0, 0}, {256, 0, 0}};
        for (int v = 1; v < dslash_variants(op->prec); v++) cand.push_back({128, v, 0});
    }
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) return cuda_error(e, "autotune events");
    float best = 1e30f;
    std::array<int, 3> pick = {op->block, op->variant, op->tensor_cores};
    const int reps = op->prec == 32 ? 10 : 3;
    int rc = GBDS_SUCCESS;
    for (const auto &c : cand) {
        op->block = c[0];
        op->variant = c[1];
        rc = gbds_op_set_tensor_cores(op, c[2]);
        if (rc == GBDS_SUCCESS) rc = gbds_op_dslash(op, gauge, psi, res, 1, 0, stream);  // warm-up
        if (rc != GBDS_SUCCESS) break;
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps; r++) gbds_op_dslash(op, gauge, psi, res, (r & 1) ? -1 : 1, 0, stream);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) break;
        if (c[2]) {
            rc = gbds_op_check(op);  // a timed-out tensor-core wait disqualifies the candidate
            if (rc != GBDS_SUCCESS) break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; pick = c; }
    }
    if (e == cudaSuccess && rc == GBDS_SUCCESS) {
        op->block = pick[0];
        op->variant = pick[1];
        rc = gbds_op_set_tensor_cores(op, pick[2]);
    }
    // the site order of the multi-RHS CUDA-core kernels: the natural order
    // and z slabs of Lz/8 planes and up (divisors of Lz), for the kernel
    // picked above
    const short zstart = op->g.zblock;
    int zpick = zstart;
    if (e == cudaSuccess && rc == GBDS_SUCCESS && generic(op) && !op->tensor_cores) {
        const int Lz = op->g.L[2];
        std::vector<int> zc = {0};
        for (int b = 2; b < Lz && b < 32768; b++)
            if (Lz % b == 0 && 8 * b >= Lz) zc.push_back(b);
        float zbest = 1e30f;
        for (int zb : zc) {
            op->g.zblock = (short)zb;
            rc = gbds_op_dslash(op, gauge, psi, res, 1, 0, stream);  // warm-up
            if (rc != GBDS_SUCCESS) break;
            cudaEventRecord(e0, s);
            for (int r = 0; r < reps; r++) gbds_op_dslash(op, gauge, psi, res, (r & 1) ? -1 : 1, 0, stream);
            cudaEventRecord(e1, s);
            e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < zbest) { zbest = ms; zpick = zb; }
        }
        // on an error the operator keeps the order it came with
        op->g.zblock = (e == cudaSuccess && rc == GBDS_SUCCESS) ? (short)zpick : zstart;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_error(e, "autotune");
    if (rc != GBDS_SUCCESS) return rc;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = {pick[0], pick[1], pick[2], zpick};
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_get_tuning(gbds_op op, int *threads, int *variant) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (threads) *threads = op->block;
    if (variant) *variant = op->variant;
    return GBDS_SUCCESS;
}

extern "C" int gbds_op_pack_gauge(gbds_op op, const void *u_packed, void *gauge, void *stream) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (!u_packed || !gauge) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    if (!aligned16(gauge)) return set_error(GBDS_ERROR_INVALID_VALUE, "gauge must be 16-byte aligned");
    if (reinterpret_cast<uintptr_t>(u_packed) & 7u)
        return set_error(GBDS_ERROR_INVALID_VALUE, "u_packed must be 8-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = launch_pack_gauge(op->g, op->prec, op->recon, u_packed, op->d_site_table, gauge, st);
    // double-float: the packed FP64 field converted in place, 16 bytes a complex
    if (e == cudaSuccess && double_float(op)) e = launch_f64_to_df(gauge, gauge, gbds_op_gauge_bytes(op) / 16, st);
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "pack_gauge");
}

extern "C" int gbds_op_pack_spinor(gbds_op op, const void *psi_packed, int parity, void *spinor, void *stream) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (!psi_packed || !spinor) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    if (parity != 0 && parity != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "parity must be 0 or 1");
    if (!aligned16(psi_packed) || !aligned16(spinor)) return set_error(GBDS_ERROR_INVALID_VALUE, "fields must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (generic(op)) {
        const float *src = static_cast<const float *>(psi_packed);
        cudaError_t e =
            op->format == GBDS_SPINOR_NATIVE
                ? launch_pack_gen_f32(op->g, op->nrhs, src, op->d_site_table, parity, spinor, st)
                : op->format == GBDS_SPINOR_F32_PAIRS
                      ? launch_pack_gen_f32p(op->g, op->nrhs, src, op->d_site_table, parity, spinor, st)
                      : launch_pack_gen_half(op->format, op->g, op->nrhs, src, op->d_site_table, parity, spinor, st);
        return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "pack_spinor");
    }
    cudaError_t e =
        launch_pack_spinor(op->g, op->prec, psi_packed, op->d_site_table, 0, parity, spinor, st, double_float(op));
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "pack_spinor");
}

extern "C" int gbds_op_unpack_spinor(gbds_op op, const void *spinor, int parity, void *psi_packed, void *stream) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (!psi_packed || !spinor) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    if (parity != 0 && parity != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "parity must be 0 or 1");
    if (!aligned16(psi_packed) || !aligned16(spinor)) return set_error(GBDS_ERROR_INVALID_VALUE, "fields must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (generic(op)) {
        float *dst = static_cast<float *>(psi_packed);
        cudaError_t e =
            op->format == GBDS_SPINOR_NATIVE
                ? launch_unpack_gen_f32(op->g, op->nrhs, spinor, op->d_site_table, parity, dst, st)
                : op->format == GBDS_SPINOR_F32_PAIRS
                      ? launch_unpack_gen_f32p(op->g, op->nrhs, spinor, op->d_site_table, parity, dst, st)
                      : launch_unpack_gen_half(op->format, op->g, op->nrhs, spinor, op->d_site_table, parity, dst, st);
        return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "unpack_spinor");
    }
    cudaError_t e =
        launch_unpack_spinor(op->g, op->prec, spinor, op->d_site_table, 0, parity, psi_packed, st, double_float(op));
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "unpack_spinor");
}

extern "C" int gbds_op_dslash(gbds_op op, const void *gauge, const void *psi, void *res, int isign, int cb,
                              void *stream) {
    if (!op) return set_error(GBDS_ERROR_NOT_INITIALIZED, "op is NULL");
    if (isign != 1 && isign != -1) return GBDS_SUCCESS;  // reference: silent no-op
    if (cb != 0 && cb != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "cb must be 0 or 1");
    if (!gauge || !psi || !res) return set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
    if (!aligned16(gauge) || !aligned16(psi) || !aligned16(res))
        return set_error(GBDS_ERROR_INVALID_VALUE, "fields must be 16-byte aligned");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (generic(op) && op->tensor_cores) {
        cudaError_t e = launch_gen_tc(op->format, op->g, op->recon, op->nrhs, gauge, psi, res, isign, cb, op->d_err, s);
        return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "dslash (tensor cores)");
    }
    if (generic(op)) {
        cudaError_t e =
            op->format == GBDS_SPINOR_NATIVE
                ? launch_gen_f32(op->g, op->recon, op->nrhs, gauge, psi, res, isign, cb, nullptr, 0.f, nullptr, s,
                                 op->variant)
                : op->format == GBDS_SPINOR_F32_PAIRS
                      ? launch_gen_f32p(op->g, op->recon, op->nrhs, gauge, psi, res, isign, cb, nullptr, 0.f, nullptr, s,
                                        op->variant)
                      : launch_gen_half(op->format, op->g, op->recon, op->nrhs, gauge, psi, res, isign, cb, nullptr, 0.f,
                                        nullptr, s, op->variant);
        return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "dslash");
    }
    cudaError_t e =
        op->prec == 32
            ? launch_dslash_f32(op->g, op->recon, gauge, psi, res, isign, cb, op->block, op->variant, s)
            : (double_float(op) ? launch_dslash_df(op->g, op->recon, gauge, psi, res, isign, cb, op->block, op->variant, s)
                                : launch_dslash_f64(op->g, op->recon, gauge, psi, res, isign, cb, op->block, op->variant, s));
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "dslash");
}

// ---------------------------------------------------------------------------
// Legacy host-pointer path (the reference's entry points)
// ---------------------------------------------------------------------------

namespace {

struct LegacyCtx {
    int refcount = 0;
    gbds_op op = nullptr;
    bool canonical = true;
    cudaStream_t stream = nullptr;
    void *d_u_packed = nullptr;    // V*4*18 reals
    void *d_gauge = nullptr;       // internal layout
    void *d_psi_packed = nullptr;  // canonical: Vh*24 reals, else V*24
    void *d_res_packed = nullptr;  // canonical: Vh*24 reals, else V*24
    void *d_psi = nullptr;         // internal, one checkerboard
    void *d_res = nullptr;         // internal, one checkerboard
    const void *cached_u = nullptr;
};

LegacyCtx g_legacy[2][2];  // [prec 32 -> 0, 64 -> 1][nd 4 -> 0, 3 -> 1]
int g_exit_on_error = 1;
int g_gauge_cache = 0;
int g_legacy_recon = 18;
int g_host_access = 0;  // 0: read/write host arrays directly where the GPU can; 1: always stage
int g_last_path = -1;   // 0 staged, 1 direct

// Address under which kernels can use a caller array, or nullptr when the
// GPU cannot reach it directly.  Pinned / registered host memory has a device
// view; on a coherent host (NVLink-C2C with address translation services) the
// GPU reads pageable memory through the host page tables; device and managed
// pointers are usable as they are.
const void *device_view(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    switch (a.type) {
    case cudaMemoryTypeDevice:
    case cudaMemoryTypeManaged: return p;
    case cudaMemoryTypeHost: return a.devicePointer;
    default: break;
    }
    int dev = 0, pageable = 0, ats = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    return (pageable && ats) ? p : nullptr;
}

LegacyCtx &ctx_for(int prec, int nd) { return g_legacy[prec == 32 ? 0 : 1][nd == 4 ? 0 : 1]; }

void legacy_release(LegacyCtx &c) {
    if (c.stream) cudaStreamSynchronize(c.stream);
    void *bufs[] = {c.d_u_packed, c.d_gauge, c.d_psi_packed, c.d_res_packed, c.d_psi, c.d_res};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (c.stream) cudaStreamDestroy(c.stream);
    gbds_op_destroy(c.op);
    c = LegacyCtx();
}

// Print and either exit(1) (the reference's behaviour) or return.
void legacy_fail(const char *fn, const std::string &msg) {
    fprintf(stderr, "%s: %s\n", fn, msg.c_str());
    if (g_exit_on_error) exit(1);
}

void legacy_init(int prec, int nd, const int *latt_size, void (*getSiteCoords)(int[], int, int),
                 int (*getLinearSiteIndex)(const int[]), const char *fn) {
    LegacyCtx &c = ctx_for(prec, nd);
    // Refcounted: a second init only increments and the first lattice stays
    // (lib/sse_su3dslash_32bit_scalar.c:95-99).
    if (c.refcount > 0) {
        c.refcount++;
        return;
    }
    if (!latt_size || !getLinearSiteIndex) {
        legacy_fail(fn, "latt_size and getLinearSiteIndex must not be NULL");
        return;
    }
    for (int mu = 0; mu < nd; mu++) {
        if (latt_size[mu] % 2 != 0) {
            char b[256];
            snprintf(b, sizeof b,
                     "This is a Dslash with checkerboarding in %d dimensions. Each GLOBAL dimension%s must be "
                     "even. Your lattice is not like this: latt_size[%d]=%d",
                     nd, nd == 3 ? " 0,1,2 (x,y,z)" : "", mu, latt_size[mu]);
            legacy_fail(fn, b);
            return;
        }
    }
    Geom g;
    if (make_geom(latt_size, nd, &g) != GBDS_SUCCESS) {
        legacy_fail(fn, g_last_error);
        return;
    }
    // The caller's layout, read through its callbacks once, here, like the
    // reference's site table (lib/shift_tables_scalar.c:240-263).
    std::vector<int> table(g.V);
    std::vector<char> seen(g.V, 0);
    bool canonical = true;
    for (int i = 0; i < g.V; i++) {
        int coord[4];
        internal_coords(g, i, coord);
        const int lin = getLinearSiteIndex(coord);
        if (lin < 0 || lin >= g.V || seen[lin]) {
            legacy_fail(fn, "getLinearSiteIndex is not a one-to-one map of the lattice onto [0, V)");
            return;
        }
        seen[lin] = 1;
        table[i] = lin;
        canonical &= (lin == i);
        if (getSiteCoords) {
            int back[4] = {-1, -1, -1, -1};
            getSiteCoords(back, 0, lin);
            if (back[0] != coord[0] || back[1] != coord[1] || back[2] != coord[2] || back[3] != coord[3]) {
                legacy_fail(fn, "getSiteCoords is not the inverse of getLinearSiteIndex");
                return;
            }
        }
    }
    LegacyCtx n;
    int rc = gbds_op_create(&n.op, latt_size, nd, prec, g_legacy_recon);
    if (rc == GBDS_SUCCESS && !canonical) rc = gbds_op_set_layout(n.op, table.data(), g.V);
    if (rc != GBDS_SUCCESS) {
        std::string m = g_last_error;
        legacy_release(n);
        legacy_fail(fn, m);
        return;
    }
    n.canonical = canonical;
    const size_t real = prec == 32 ? 4 : 8;
    const size_t spin_sites = canonical ? (size_t)g.Vh : (size_t)g.V;
    cudaError_t e = cudaStreamCreateWithFlags(&n.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&n.d_u_packed, (size_t)g.V * 4 * 18 * real);
    if (e == cudaSuccess) e = cudaMalloc(&n.d_gauge, gbds_op_gauge_bytes(n.op));
    if (e == cudaSuccess) e = cudaMalloc(&n.d_psi_packed, spin_sites * 24 * real);
    if (e == cudaSuccess) e = cudaMalloc(&n.d_res_packed, spin_sites * 24 * real);
    if (e == cudaSuccess) e = cudaMalloc(&n.d_psi, gbds_op_spinor_bytes(n.op));
    if (e == cudaSuccess) e = cudaMalloc(&n.d_res, gbds_op_spinor_bytes(n.op));
    if (e != cudaSuccess) {
        cuda_error(e, "legacy init");
        std::string m = g_last_error;
        legacy_release(n);
        legacy_fail(fn, m);
        return;
    }
    n.refcount = 1;
    c = n;
}

void legacy_free(int prec, int nd) {
    LegacyCtx &c = ctx_for(prec, nd);
    if (c.refcount == 0) return;
    if (--c.refcount == 0) legacy_release(c);
}

void legacy_apply(int prec, int nd, const void *u, const void *psi, void *res, int isign, int cb, const char *fn) {
    LegacyCtx &c = ctx_for(prec, nd);
    if (isign != 1 && isign != -1) return;  // lib/sse_su3dslash_32bit_scalar.c:162-179
    if (c.refcount == 0) {
        fprintf(stderr, "%s: called before init; nothing done\n", fn);
        return;
    }
    if (cb != 0 && cb != 1) {
        fprintf(stderr, "%s: cb must be 0 or 1 (got %d); nothing done\n", fn, cb);
        return;
    }
    if (!u || !psi || !res) {
        fprintf(stderr, "%s: NULL field pointer; nothing done\n", fn);
        return;
    }
    const Geom &g = c.op->g;
    const size_t real = prec == 32 ? 4 : 8;
    const size_t spinor = 24 * real;
    const int target = 1 - cb;
    cudaStream_t s = c.stream;
    const int *table = c.op->d_site_table;
    cudaError_t e = cudaSuccess;
    const bool reuse_gauge = g_gauge_cache && c.cached_u == u;
    const void *du = nullptr, *dpsi = nullptr;
    void *dres = nullptr;
    if (c.canonical && g_host_access == 0) {
        du = reuse_gauge ? u : device_view(u);
        dpsi = device_view(psi);
        dres = const_cast<void *>(device_view(res));
    }
    const bool aligned = ((reinterpret_cast<uintptr_t>(du) | reinterpret_cast<uintptr_t>(dpsi) |
                           reinterpret_cast<uintptr_t>(dres)) & 15u) == 0;
    if (du && dpsi && dres && aligned) {
        // Direct: the layout kernels read u and psi and write res where they
        // lie, with no intermediate copy.
        if (!reuse_gauge) {
            e = launch_pack_gauge(g, prec, c.op->recon, du, nullptr, c.d_gauge, s);
            c.cached_u = e == cudaSuccess ? u : nullptr;
        }
        if (e == cudaSuccess) e = launch_pack_spinor(g, prec, dpsi, nullptr, 0, cb, c.d_psi, s);
        if (e == cudaSuccess)
            e = prec == 32 ? launch_dslash_f32(g, c.op->recon, c.d_gauge, c.d_psi, c.d_res, isign, cb, c.op->block, c.op->variant, s)
                           : launch_dslash_f64(g, c.op->recon, c.d_gauge, c.d_psi, c.d_res, isign, cb, c.op->block, c.op->variant, s);
        if (e == cudaSuccess) e = launch_unpack_spinor(g, prec, c.d_res, nullptr, 0, target, dres, s);
        cudaError_t e2 = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = e2;
        g_last_path = 1;
        if (e != cudaSuccess) {
            c.cached_u = nullptr;
            fprintf(stderr, "%s: CUDA error: %s\n", fn, cudaGetErrorString(e));
        }
        return;
    }
    g_last_path = 0;
    if (!reuse_gauge) {
        e = cudaMemcpyAsync(c.d_u_packed, u, (size_t)g.V * 4 * 18 * real, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_pack_gauge(g, prec, c.op->recon, c.d_u_packed, table, c.d_gauge, s);
        c.cached_u = e == cudaSuccess ? u : nullptr;
    }
    if (c.canonical) {
        // Checkerboards are contiguous halves of the caller's arrays.
        const char *src = static_cast<const char *>(psi) + (size_t)cb * g.Vh * spinor;
        if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_psi_packed, src, (size_t)g.Vh * spinor, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_pack_spinor(g, prec, c.d_psi_packed, nullptr, cb * g.Vh, cb, c.d_psi, s);
        if (e == cudaSuccess)
            e = prec == 32 ? launch_dslash_f32(g, c.op->recon, c.d_gauge, c.d_psi, c.d_res, isign, cb, c.op->block, c.op->variant, s)
                           : launch_dslash_f64(g, c.op->recon, c.d_gauge, c.d_psi, c.d_res, isign, cb, c.op->block, c.op->variant, s);
        if (e == cudaSuccess) e = launch_unpack_spinor(g, prec, c.d_res, nullptr, target * g.Vh, target, c.d_res_packed, s);
        char *dst = static_cast<char *>(res) + (size_t)target * g.Vh * spinor;
        if (e == cudaSuccess) e = cudaMemcpyAsync(dst, c.d_res_packed, (size_t)g.Vh * spinor, cudaMemcpyDeviceToHost, s);
    } else {
        // Arbitrary layout: whole arrays move; sites of the other checkerboard
        // of `res` are carried through unchanged.
        if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_psi_packed, psi, (size_t)g.V * spinor, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_res_packed, res, (size_t)g.V * spinor, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_pack_spinor(g, prec, c.d_psi_packed, table, 0, cb, c.d_psi, s);
        if (e == cudaSuccess)
            e = prec == 32 ? launch_dslash_f32(g, c.op->recon, c.d_gauge, c.d_psi, c.d_res, isign, cb, c.op->block, c.op->variant, s)
                           : launch_dslash_f64(g, c.op->recon, c.d_gauge, c.d_psi, c.d_res, isign, cb, c.op->block, c.op->variant, s);
        if (e == cudaSuccess) e = launch_unpack_spinor(g, prec, c.d_res, table, 0, target, c.d_res_packed, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(res, c.d_res_packed, (size_t)g.V * spinor, cudaMemcpyDeviceToHost, s);
    }
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) {
        c.cached_u = nullptr;
        fprintf(stderr, "%s: CUDA error: %s\n", fn, cudaGetErrorString(e));
    }
}

// Reorder the gauge field from SZIN order u[mu][cb][site] to u_tmp[cb][site][mu]
// (no transpose), as lib/packer_nopad.c:29-45 does.  `volume` is the number of
// sites per checkerboard.
template <typename R>
void pack_gauge_field_t(int volume, R *u, R *u_tmp) {
    if (volume <= 0 || !u || !u_tmp) return;
    const size_t m = 18;
    for (int cb = 0; cb < 2; cb++)
        for (int ix = 0; ix < volume; ix++)
            for (int mu = 0; mu < 4; mu++)
                memcpy(u_tmp + m * (mu + 4 * ((size_t)ix + (size_t)volume * cb)),
                       u + m * ((size_t)ix + (size_t)volume * (cb + 2 * mu)), m * sizeof(R));
}

// The reference's unpack_gauge_field (lib/packer_nopad.c:47-69) copies u_tmp
// to u with the same index on both sides (it is not the inverse of
// pack_gauge_field); kept as such for callers that rely on it.
template <typename R>
void unpack_gauge_field_t(int volume, R *u_tmp, R *u) {
    if (volume <= 0 || !u || !u_tmp) return;
    memmove(u, u_tmp, (size_t)8 * volume * 18 * sizeof(R));
}

}  // namespace

#define GBDS_LEGACY_ENTRY(P, R, SUF)                                                                        \
    extern "C" void gbds_sse_init##SUF(const int *l, void (*gc)(int[], int, int), int (*gl)(const int[]),   \
                                       int (*nn)(const int[])) {                                            \
        (void)nn;                                                                                           \
        legacy_init(P, 4, l, gc, gl, "init_sse_su3dslash");                                                 \
    }                                                                                                       \
    extern "C" void gbds_sse_free##SUF(void) { legacy_free(P, 4); }                                         \
    extern "C" void gbds_sse_wilson##SUF(R *u, R *psi, R *res, int isign, int cb) {                         \
        legacy_apply(P, 4, u, psi, res, isign, cb, "sse_su3dslash_wilson");                                 \
    }                                                                                                       \
    extern "C" void gbds_sse_init_3d##SUF(const int *l, void (*gc)(int[], int, int), int (*gl)(const int[]), \
                                          int (*nn)(const int[])) {                                         \
        (void)nn;                                                                                           \
        legacy_init(P, 3, l, gc, gl, "init_sse_su3dslash_3d");                                              \
    }                                                                                                       \
    extern "C" void gbds_sse_free_3d##SUF(void) { legacy_free(P, 3); }                                      \
    extern "C" void gbds_sse_wilson_3d##SUF(R *u, R *psi, R *res, int isign, int cb) {                      \
        legacy_apply(P, 3, u, psi, res, isign, cb, "sse_su3dslash_wilson_3d");                              \
    }                                                                                                       \
    extern "C" void gbds_pack_gauge_field##SUF(int volume, R *u, R *u_tmp) { pack_gauge_field_t(volume, u, u_tmp); } \
    extern "C" void gbds_unpack_gauge_field##SUF(int volume, R *u_tmp, R *u) { unpack_gauge_field_t(volume, u_tmp, u); }

GBDS_LEGACY_ENTRY(32, float, _f32)
GBDS_LEGACY_ENTRY(64, double, _f64)

extern "C" int gbds_legacy_set_exit_on_error(int on) {
    g_exit_on_error = on ? 1 : 0;
    return GBDS_SUCCESS;
}

extern "C" int gbds_legacy_set_gauge_cache(int on) {
    g_gauge_cache = on ? 1 : 0;
    for (auto &a : g_legacy)
        for (auto &c : a) c.cached_u = nullptr;
    return GBDS_SUCCESS;
}

extern "C" int gbds_legacy_invalidate_gauge(void) {
    for (auto &a : g_legacy)
        for (auto &c : a) c.cached_u = nullptr;
    return GBDS_SUCCESS;
}

extern "C" int gbds_legacy_set_recon(int recon) {
    if (recon != 18 && recon != 12) return set_error(GBDS_ERROR_INVALID_VALUE, "recon must be 18 or 12");
    g_legacy_recon = recon;
    return GBDS_SUCCESS;
}

extern "C" int gbds_legacy_set_host_access(int mode) {
    if (mode != 0 && mode != 1) return set_error(GBDS_ERROR_INVALID_VALUE, "mode must be 0 (direct where possible) or 1 (staged)");
    g_host_access = mode;
    return GBDS_SUCCESS;
}

extern "C" int gbds_legacy_last_path(void) { return g_last_path; }

extern "C" int gbds_legacy_refcount(int prec, int nd) {
    if ((prec != 32 && prec != 64) || (nd != 3 && nd != 4)) return -1;
    return ctx_for(prec, nd).refcount;
}

// ---------------------------------------------------------------------------
// QDP++ cb2 / cb3d callbacks (the internal order, so no permutation results)
// ---------------------------------------------------------------------------

namespace {
Geom g_layout_geom = {{2, 2, 2, 2}, 4, 1, 16, 8, 64};
}

extern "C" int gbds_layout_select(int nd, const int dims[4]) {
    Geom g;
    int rc = make_geom(dims, nd, &g);
    if (rc == GBDS_SUCCESS) g_layout_geom = g;
    return rc;
}

extern "C" void gbds_layout_site_coords(int coord[], int node, int linearsite) {
    (void)node;
    internal_coords(g_layout_geom, linearsite, coord);
}

extern "C" int gbds_layout_linear_site_index(const int coord[]) {
    const Geom &g = g_layout_geom;
    if (g.nd == 4) {
        const int p = (coord[0] + coord[1] + coord[2] + coord[3]) & 1;
        return p * g.Vh + ((coord[3] * g.L[2] + coord[2]) * g.L[1] + coord[1]) * g.Lxh + coord[0] / 2;
    }
    const int p = (coord[0] + coord[1] + coord[2]) & 1;
    return p * g.Vh + coord[3] + g.L[3] * (coord[0] / 2 + g.Lxh * (coord[1] + g.L[1] * coord[2]));
}

extern "C" int gbds_layout_node_number(const int coord[]) {
    (void)coord;
    return 0;
}
