// Uneven batches: several lattices, each with its own gauge field, spinors and
// number of right-hand sides, applied in ONE persistent kernel launch.
//
// The (site, rhs) pairs of every lattice are cut into tiles of blockDim.x
// threads; a work list of tiles is built once on the host; each CTA of a
// grid sized to the machine walks the list with a fixed stride (no atomics,
// no waiting on other CTAs), so the launch can be captured in a CUDA graph
// and replayed.  The autotuner picks the tile size, the number of resident
// CTAs and the order of the work list.  FP32 arithmetic and links; spinor
// storage FP32 / bfloat16 / half + norm; 4D operator.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "dslash_gen.cuh"

namespace gbds {
namespace {

struct Problem {
    Geom g;
    int nrhs;
    int isign;
    int pt;
    size_t link_block_bytes;
    size_t cs;
    const char *gauge;
    const char *psi;
    char *res;
};

struct Tile {
    int problem;
    int first;  // first (site, rhs) index
    int end;
};

// Lattice descriptors travel by value in the kernel parameters (the constant
// bank: one broadcast read per warp), not through global memory.
constexpr int kMaxBatch = 32;
struct BatchParams {
    int n;
    Problem p[kMaxBatch];
};

template <int FMT, int RECON, int ISIGN, int NRHS, int MU>
__device__ __forceinline__ void batch_hop_pair(const Problem &P, int h, int r, const Nbr &n, cx<float> (&acc)[4][3]) {
    const int ps = 1 - P.pt;
    const int nr = NRHS > 0 ? NRHS : P.nrhs;
    cx<float> s[4][3], hs[2][3], w[2][3], U[3][3];
    Sio<FMT>::load(P.psi, P.cs, (size_t)n.f[MU] * nr + r, s);
    Field<float>::template load_link<RECON>(P.gauge + (size_t)(P.pt * 4 + MU) * P.link_block_bytes, P.g.stride, h, U);
    project<MU, ISIGN>(s, hs);
    su3_mul<false>(U, hs, w);
    reconstruct<MU, ISIGN>(acc, w);
    Sio<FMT>::load(P.psi, P.cs, (size_t)n.b[MU] * nr + r, s);
    Field<float>::template load_link<RECON>(P.gauge + (size_t)(ps * 4 + MU) * P.link_block_bytes, P.g.stride, n.b[MU], U);
    project<MU, -ISIGN>(s, hs);
    su3_mul<true>(U, hs, w);
    reconstruct<MU, -ISIGN>(acc, w);
}

template <int FMT, int RECON, int ISIGN, int NRHS>
__device__ __forceinline__ void batch_site(const Problem &P, int t) {
    const int nr = NRHS > 0 ? NRHS : P.nrhs;
    const int h = t / nr, r = t - h * nr;
    Nbr n;
    neighbours<4>(P.g, h, P.pt, n);
    cx<float> acc[4][3];
#pragma unroll
    for (int s = 0; s < 4; s++)
#pragma unroll
        for (int c = 0; c < 3; c++) acc[s][c] = {0.f, 0.f};
    batch_hop_pair<FMT, RECON, ISIGN, NRHS, 0>(P, h, r, n, acc);
    batch_hop_pair<FMT, RECON, ISIGN, NRHS, 1>(P, h, r, n, acc);
    batch_hop_pair<FMT, RECON, ISIGN, NRHS, 2>(P, h, r, n, acc);
    batch_hop_pair<FMT, RECON, ISIGN, NRHS, 3>(P, h, r, n, acc);
    Sio<FMT>::store(P.res, P.cs, (size_t)h * nr + r, acc);
}


template <int FMT, int RECON>
__global__ void __launch_bounds__(256, 3) batch_kernel(const __grid_constant__ BatchParams bp, const Tile *__restrict__ tiles,
                                                    int ntiles) {
    pdl_allow_next();
    pdl_wait_prev();
    for (int w = blockIdx.x; w < ntiles; w += gridDim.x) {
        const Tile tl = tiles[w];
        const Problem &P = bp.p[tl.problem];
        const int t = tl.first + threadIdx.x;
        if (t < tl.end) {
            // the count of right-hand sides stays a run-time value: one body
            // per isign keeps the register budget of the single-lattice kernel
            if (P.isign > 0) batch_site<FMT, RECON, 1, 0>(P, t);
            else batch_site<FMT, RECON, -1, 0>(P, t);
        }
    }
}

}  // namespace
}  // namespace gbds

using namespace gbds;

struct gbds_batch_s {
    std::vector<Problem> probs;
    int recon = 18;
    int format = 0;
    int block = 128;     // threads per tile
    int grid = 0;        // resident CTAs (0: one per tile up to the machine size)
    int order = 0;       // 0: tiles of one lattice after another; 1: interleaved across lattices
    BatchParams params;
    Tile *d_tiles = nullptr;
    int ntiles = 0;
    int sms = 0;
    cudaGraphExec_t graph = nullptr;
};

namespace {

int build_tiles(gbds_batch b) {
    std::vector<std::vector<Tile>> per(b->probs.size());
    for (size_t p = 0; p < b->probs.size(); p++) {
        const int n = b->probs[p].g.Vh * b->probs[p].nrhs;
        for (int f = 0; f < n; f += b->block) per[p].push_back({(int)p, f, std::min(n, f + b->block)});
    }
    std::vector<Tile> all;
    if (b->order == 0) {
        for (auto &v : per) all.insert(all.end(), v.begin(), v.end());
    } else {
        // round-robin over lattices, proportional to their sizes
        size_t left = 0;
        for (auto &v : per) left += v.size();
        std::vector<size_t> next(per.size(), 0);
        while (left) {
            size_t best = 0;
            double bp = 1e300;
            for (size_t p = 0; p < per.size(); p++) {
                if (next[p] >= per[p].size()) continue;
                const double key = (next[p] + 0.5) / per[p].size();
                if (key < bp) { bp = key; best = p; }
            }
            all.push_back(per[best][next[best]++]);
            left--;
        }
    }
    if (b->d_tiles) cudaFree(b->d_tiles);
    b->d_tiles = nullptr;
    b->ntiles = (int)all.size();
    cudaError_t e = cudaMalloc(&b->d_tiles, sizeof(Tile) * all.size());
    if (e == cudaSuccess) e = cudaMemcpy(b->d_tiles, all.data(), sizeof(Tile) * all.size(), cudaMemcpyHostToDevice);
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "batch tiles");
}

cudaError_t launch_batch(gbds_batch b, cudaStream_t st) {
    int grid = b->grid > 0 ? b->grid : b->ntiles;
    grid = std::max(1, std::min(grid, b->ntiles));
#define GBDS_B(F, R) launch_pdl(batch_kernel<F, R>, dim3(grid), b->block, st, b->params, (const Tile *)b->d_tiles, b->ntiles)
    if (b->recon == 18) {
        if (b->format == 0) GBDS_B(kFmtNative, 18); else if (b->format == 1) GBDS_B(kFmtBF16, 18);
        else if (b->format == 2) GBDS_B(kFmtF16N, 18); else GBDS_B(kFmtF32Pairs, 18);
    } else {
        if (b->format == 0) GBDS_B(kFmtNative, 12); else if (b->format == 1) GBDS_B(kFmtBF16, 12);
        else if (b->format == 2) GBDS_B(kFmtF16N, 12); else GBDS_B(kFmtF32Pairs, 12);
    }
#undef GBDS_B
    count_launch();
    return cudaGetLastError();
}

}  // namespace

extern "C" int gbds_batch_create(gbds_batch *out, const gbds_batch_item *items, int n, int recon, int format) {
    if (!out || !items || n <= 0) return set_error(GBDS_ERROR_INVALID_VALUE, "need at least one batch item");
    if (n > kMaxBatch) return set_error(GBDS_ERROR_INVALID_VALUE, "at most 32 lattices per batch");
    *out = nullptr;
    if (recon != 18 && recon != 12) return set_error(GBDS_ERROR_INVALID_VALUE, "recon must be 18 or 12");
    if (format < 0 || format > 3) return set_error(GBDS_ERROR_INVALID_VALUE, "unknown spinor format");
    gbds_batch b = new (std::nothrow) gbds_batch_s;
    if (!b) return set_error(GBDS_ERROR_OUT_OF_MEMORY, "host allocation failed");
    b->recon = recon;
    b->format = format;
    for (int i = 0; i < n; i++) {
        const gbds_batch_item &it = items[i];
        Problem P;
        int rc = make_geom(it.dims, 4, &P.g);
        if (rc == GBDS_SUCCESS && (it.nrhs < 1 || it.nrhs > 32)) rc = set_error(GBDS_ERROR_INVALID_VALUE, "nrhs must be in [1, 32]");
        if (rc == GBDS_SUCCESS && it.isign != 1 && it.isign != -1) rc = set_error(GBDS_ERROR_INVALID_VALUE, "isign must be +1 or -1");
        if (rc == GBDS_SUCCESS && it.cb != 0 && it.cb != 1) rc = set_error(GBDS_ERROR_INVALID_VALUE, "cb must be 0 or 1");
        if (rc == GBDS_SUCCESS && (!it.gauge || !it.psi || !it.res)) rc = set_error(GBDS_ERROR_INVALID_VALUE, "NULL field pointer");
        if (rc != GBDS_SUCCESS) {
            delete b;
            return rc;
        }
        P.nrhs = it.nrhs;
        P.isign = it.isign;
        P.pt = 1 - it.cb;
        P.link_block_bytes = (size_t)recon * 4 * P.g.stride;
        P.cs = (size_t)P.g.stride * it.nrhs;
        P.gauge = static_cast<const char *>(it.gauge);
        P.psi = static_cast<const char *>(it.psi);
        P.res = static_cast<char *>(it.res);
        b->probs.push_back(P);
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    b->grid = b->sms * 4;
    b->params.n = n;
    for (int i = 0; i < n; i++) b->params.p[i] = b->probs[i];
    int rc = build_tiles(b);
    if (rc != GBDS_SUCCESS) {
        gbds_batch_destroy(b);  // frees a tile list that was allocated before the failing copy
        return rc;
    }
    *out = b;
    return GBDS_SUCCESS;
}

extern "C" int gbds_batch_destroy(gbds_batch b) {
    if (!b) return GBDS_SUCCESS;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->d_tiles) cudaFree(b->d_tiles);
    delete b;
    return GBDS_SUCCESS;
}

extern "C" int gbds_batch_set_schedule(gbds_batch b, int tile_threads, int resident_ctas, int order) {
    if (!b) return set_error(GBDS_ERROR_NOT_INITIALIZED, "batch is NULL");
    if (tile_threads < 32 || tile_threads > 256 || tile_threads % 32)
        return set_error(GBDS_ERROR_INVALID_VALUE, "tile_threads must be a multiple of 32 in [32, 256]");
    if (resident_ctas < 0 || (order != 0 && order != 1)) return set_error(GBDS_ERROR_INVALID_VALUE, "bad schedule");
    b->block = tile_threads;
    b->grid = resident_ctas;
    b->order = order;
    return build_tiles(b);
}

extern "C" int gbds_batch_get_schedule(gbds_batch b, int *tile_threads, int *resident_ctas, int *order, int *ntiles) {
    if (!b) return set_error(GBDS_ERROR_NOT_INITIALIZED, "batch is NULL");
    if (tile_threads) *tile_threads = b->block;
    if (resident_ctas) *resident_ctas = b->grid;
    if (order) *order = b->order;
    if (ntiles) *ntiles = b->ntiles;
    return GBDS_SUCCESS;
}

extern "C" int gbds_batch_launch(gbds_batch b, void *stream) {
    if (!b) return set_error(GBDS_ERROR_NOT_INITIALIZED, "batch is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = b->graph ? cudaGraphLaunch(b->graph, st) : launch_batch(b, st);
    if (b->graph && e == cudaSuccess) count_launch();
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "gbds_batch_launch");
}

extern "C" int gbds_batch_capture_graph(gbds_batch b, void *stream) {
    if (!b) return set_error(GBDS_ERROR_NOT_INITIALIZED, "batch is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!st) return set_error(GBDS_ERROR_INVALID_VALUE, "graph capture needs a non-default stream");
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t le = launch_batch(b, st);
        e = cudaStreamEndCapture(st, &g);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    return e == cudaSuccess ? GBDS_SUCCESS : cuda_error(e, "gbds_batch_capture_graph");
}

extern "C" int gbds_batch_autotune(gbds_batch b, void *stream) {
    if (!b) return set_error(GBDS_ERROR_NOT_INITIALIZED, "batch is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int pick[3] = {b->block, b->grid, b->order};
    cudaError_t e = cudaSuccess;
    // every (tile size, resident CTAs, order) candidate; the first CUDA error
    // ends the whole search
    for (int blk : {64, 128, 256}) {
        for (int mult : {2, 4, 6, 8}) {
            for (int order : {0, 1}) {
                int rc = gbds_batch_set_schedule(b, blk, b->sms * mult * 128 / blk, order);
                if (rc != GBDS_SUCCESS) continue;
                launch_batch(b, st);
                cudaEventRecord(e0, st);
                for (int r = 0; r < 3; r++) launch_batch(b, st);
                cudaEventRecord(e1, st);
                e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) break;
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) {
                    best = ms;
                    pick[0] = blk;
                    pick[1] = b->grid;
                    pick[2] = order;
                }
            }
            if (e != cudaSuccess) break;
        }
        if (e != cudaSuccess) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_error(e, "gbds_batch_autotune");
    return gbds_batch_set_schedule(b, pick[0], pick[1], pick[2]);
}
