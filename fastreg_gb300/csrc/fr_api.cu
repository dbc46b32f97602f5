// fr_api.cu -- host side of the C ABI (include/fastreg_gb300.h).
//
// A handle owns one packed cohort of pairs on the device (one allocation carved into
// fields), the tile table the kernels walk, and a CUDA graph holding every iteration
// of a registration.  fr_register is fr_register_batch with one pair.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fastreg_gb300.h"
#include "fr_kernels.h"
#include "fr_limits.h"
#include "fr_tma.cuh"
#include "fr_sob.h"

#include <chrono>
#include <map>
#include <mutex>

using frg::Pair;
using frg::Tile;

// The solver kernels and their tile tables.  Each kernel walks its own table of 32 x 8 x
// depth tiles with a persistent grid of blocks_per_sm x SMs blocks (capped at the tile
// count); the shape is the default below or the autotuner's choice.
enum Role { R_LAP, R_PA, R_PB, R_SG, R_SS, R_SB, R_COUNT };
struct Shape {
    int depth = 16;  // slices per tile
    int bps = 0;     // blocks per SM (-1: one block per tile, scheduled by the hardware)
    int variant = 0; // 0: staging by per-thread cp.async; 1: by TMA tensor copies (kernels that have both)
};
struct TileSet {
    Shape shape;
    std::vector<Tile> h;
    Tile* d = nullptr;  // device copy (capacity cap tiles)
    size_t cap = 0;
    int occ[2] = {1, 1};  // resident blocks per SM of each variant at its registers and shared memory
    int grid = 0;
};
// defaults (AUTOTUNE=0), the autotuner's usual choice on the 182x218x182 pair: slices per
// tile, and whether each tile is its own block (scheduled by the hardware) instead of a
// persistent grid at the occupancy limit
static const int kDefaultDepth[R_COUNT] = {16, 24, 24, 12, 32, 8};
static const bool kDefaultPerTile[R_COUNT] = {true, true, false, true, true, false};
static const int kDefaultVariant[R_COUNT] = {0, 0, 0, 0, 0, 0};
static const int kMinDepth = 1;  // thin tiles give small volumes enough blocks
static const int kTuneWarmIters = 20;  // iterations run before the autotuner times shapes

struct fr_handle {
    fr_params P;
    std::string err;
    int device = 0;
    int num_sms = 0;

    // cohort
    std::vector<std::array<int, 3>> dims;
    int npairs = 0;
    long long NT = 0;
    std::vector<Pair> hpairs;
    std::vector<Tile> htiles;  // 32 x 8 x 16 tiles of the I/O kernels
    TileSet ts[R_COUNT];       // the solver kernels' own tables
    bool tuned = false;        // the shapes of this cohort are settled
    std::vector<fr_pair> io;  // caller buffers of the current registration
    std::vector<float> pair_w_reg;  // per-pair W_REG from fr_set_pair_w_reg (empty: P.w_reg)

    // device memory
    char* block = nullptr;
    size_t block_bytes = 0;
    Pair* d_pairs = nullptr;
    Tile* d_tiles = nullptr;
    frg::PairIO* d_io = nullptr;
    float *S = nullptr, *T = nullptr;
    int16_t *labS = nullptr, *labT = nullptr;
    float *rho[2] = {nullptr, nullptr}, *v[2] = {nullptr, nullptr}, *pinv[2] = {nullptr, nullptr};
    float* psi = nullptr;
    float4* LT = nullptr;
    int* stop = nullptr;
    unsigned long long* keys = nullptr;
    unsigned long long* trace = nullptr;
    unsigned int* counter = nullptr;
    CUtensorMap* tmaps = nullptr;   // [npairs][TM_COUNT] tensor maps of the TMA-staged kernels
    unsigned int* dev_err = nullptr;  // device error word of the staged kernels
    bool tma_ok = false;            // the maps of this cohort are encoded (else only variant 0 runs)
    double* tile_partials = nullptr;
    int* pair_tiles = nullptr;  // [npairs + 1] first I/O tile of each pair
    long long* tile_folds = nullptr;
    unsigned long long* dice = nullptr;
    double* pair_energy = nullptr;
    long long* pair_folds = nullptr;
    int trace_cap = 0;  // iterations the trace array holds

    // sobolev-mode scratch
    float* grad = nullptr;  // unsmoothed gradient / smoothing temporaries (3 planes x 2)
    double* sob_energy = nullptr;

    // launch shape of the I/O kernels
    int grid_io = 0;

    // graph of all iterations of a registration
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;

    // bookkeeping
    int last_iter = 0;      // iterations enqueued in the current registration
    bool have_state = false;
    bool finished = false;
    bool stats_ready = false;
    std::vector<fr_stats> stats;
    cudaStream_t last_stream = nullptr;
};

namespace {

int fail(fr_handle* h, int code, const char* fmt, ...) {
    if (h) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        h->err = buf;
    }
    return code;
}

#define FR_CUDA(h, call)                                                                              \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return fail((h), FR_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),    \
                        __FILE__, __LINE__);                                                          \
    } while (0)

#define FR_LAUNCHED(h)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = cudaGetLastError();                                                          \
        if (e_ != cudaSuccess)                                                                        \
            return fail((h), FR_ERR_CUDA, "kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                          \
    } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// an index of the packed (row-padded) layout -> the caller's x + X*(y + Y*z)
long long user_index(const Pair& P, long long ip) {
    const long long row = ip / P.Xp, x = ip - row * P.Xp;
    return x + (long long)P.X * row;
}

// decode a max-norm key: norm and packed index (index 0 when the norm is 0)
void decode_key(unsigned long long k, float* norm, long long* ip) {
    const unsigned bits = (unsigned)(k >> 32);
    std::memcpy(norm, &bits, 4);
    *ip = bits ? (long long)(0xffffffffu - (unsigned)(k & 0xffffffffu)) : 0;
}

// t for every iteration: t = alpha, then t += alpha with the RESET_ITER restart
// (solver.cu:327-328,428-432)
std::vector<float> t_schedule(const fr_params& P) {
    std::vector<float> ts;
    ts.reserve(std::max(P.max_iter, 0));
    float t = P.alpha;
    for (int iter = 1; iter <= P.max_iter; ++iter) {
        ts.push_back(t);
        int next = iter + 1;
        t += P.alpha;
        if (P.reset_iter > 0 && next % P.reset_iter == 0) t = P.alpha;
    }
    return ts;
}

int check_params(fr_handle* h, const fr_params* p) {
    if (!p) return fail(h, FR_ERR_INVALID_ARG, "params is NULL");
    for (int c = 0; c < 3; ++c)
        if (p->volume_dims[c] < 1) return fail(h, FR_ERR_INVALID_ARG, "volume_dims[%d] = %d < 1", c, p->volume_dims[c]);
    if (p->no_labels < 1 || p->no_labels > FR_MAX_LABELS)
        return fail(h, FR_ERR_INVALID_ARG, "no_labels = %d outside [1, %d]", p->no_labels, FR_MAX_LABELS);
    if (p->max_iter < 0) return fail(h, FR_ERR_INVALID_ARG, "max_iter = %d < 0", p->max_iter);
    if (p->solver != FR_SOLVER_REFERENCE && p->solver != FR_SOLVER_SOBOLEV)
        return fail(h, FR_ERR_INVALID_ARG, "unknown solver %d", p->solver);
    if (p->solver == FR_SOLVER_REFERENCE && !(p->alpha > 0.f))
        return fail(h, FR_ERR_INVALID_ARG, "alpha must be > 0 (t starts at alpha)");
    if (p->solver == FR_SOLVER_SOBOLEV) {
        if (p->smooth_width < 1 || p->smooth_width > frg::kMaxSmoothWidth || (p->smooth_width & 1) == 0)
            return fail(h, FR_ERR_INVALID_ARG, "smooth_width = %d must be odd and in [1, %d]", p->smooth_width,
                        frg::kMaxSmoothWidth);
        if (!(p->smooth_sigma > 0.f)) return fail(h, FR_ERR_INVALID_ARG, "smooth_sigma must be > 0");
    }
    if (p->verbosity < 0 || p->verbosity > 2) return fail(h, FR_ERR_INVALID_ARG, "verbosity must be 0, 1 or 2");
    if (p->staging < 0 || p->staging > 2) return fail(h, FR_ERR_INVALID_ARG, "staging must be 0, 1 or 2");
    return FR_OK;
}

int occupancy_grid(fr_handle* h, const void* fn, int ntiles, size_t smem = 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    long long g = (long long)per_sm * h->num_sms;
    return (int)std::max(1LL, std::min<long long>(g, ntiles));
}

// The staged kernels' error word (set when a bounded wait gave up); the caller has
// synchronised the work that could set it.
int check_device_error(fr_handle* h) {
    if (!h->dev_err) return FR_OK;
    unsigned int e = 0;
    FR_CUDA(h, cudaMemcpy(&e, h->dev_err, sizeof e, cudaMemcpyDeviceToHost));
    if (e & frg::kErrTmaTimeout)
        return fail(h, FR_ERR_CUDA, "a TMA staging wait gave up after its time limit (device error word %u)", e);
    return FR_OK;
}

void release(fr_handle* h) {
    if (h->graph) cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
    h->graph_valid = false;
    if (h->block) cudaFree(h->block);
    h->block = nullptr;
    h->block_bytes = 0;
    h->npairs = 0;
    h->dims.clear();
    h->have_state = false;
}

// ---- per-kernel tile tables ----
std::vector<int> active_roles(const fr_handle* h) {
    if (h->P.solver == FR_SOLVER_REFERENCE) return {R_LAP, R_PA, R_PB};
    return {R_SG, R_SS, R_SB};
}

// kernels with a TMA-staged variant
bool has_tma_variant(int r) { return r != R_COUNT; }  // every solver kernel has one

// the staging variants kernel r may run with this handle's STAGING and cohort
std::vector<int> allowed_variants(const fr_handle* h, int r) {
    if (!has_tma_variant(r) || !h->tma_ok || h->P.staging == 1) return {0};
    if (h->P.staging == 2) return {1};
    return {0, 1};
}

const void* role_fn(const fr_handle* h, int r, int variant = 0) {
    switch (r) {
        case R_LAP: return variant ? (const void*)frg::ref_laplacian_tma_kernel : (const void*)frg::ref_laplacian_kernel;
        case R_PA: return variant ? (const void*)frg::ref_pass_a_tma_kernel : (const void*)frg::ref_pass_a_kernel;
        case R_PB: return variant ? (const void*)frg::ref_pass_b_staged_kernel : (const void*)frg::ref_pass_b_kernel;
        case R_SG: return variant ? (const void*)frg::sob_grad_tma_kernel : (const void*)frg::sob_grad_kernel;
        case R_SS: return frg::sob_smooth3_fn(h->P.smooth_width / 2, variant);
        default: return variant ? (const void*)frg::sob_pass_b_staged_kernel : (const void*)frg::sob_pass_b_kernel;
    }
}

size_t role_smem(int r, int variant = 0) {
    switch (r) {
        case R_LAP: return variant ? frg::ref_laplacian_tma_smem_bytes() : frg::ref_laplacian_smem_bytes();
        case R_PA: return variant ? frg::ref_pass_a_tma_smem_bytes() : frg::ref_pass_a_smem_bytes();
        case R_SG: return variant ? frg::sob_grad_tma_smem_bytes() : frg::sob_grad_smem_bytes();
        case R_PB:
        case R_SB: return variant ? frg::gather_staged_smem_bytes() : 0;
        default: return 0;
    }
}

// threads per block and tile rows of kernel r's variant
int role_threads(int r, int variant = 0) { return (r == R_PB && variant == 0) ? frg::kPassBThreads : 256; }
int role_tile_y(int r, int variant = 0) { return (r == R_PB && variant == 0) ? frg::kPassBTileY : frg::kTileY; }

typedef std::array<Shape, R_COUNT> Shapes;

Shapes default_shapes(const fr_handle* h) {
    Shapes sh{};
    for (int r = 0; r < R_COUNT; ++r) {
        const std::vector<int> al = allowed_variants(h, r);
        const int v = al.size() == 1 ? al[0] : kDefaultVariant[r];
        sh[r] = Shape{kDefaultDepth[r], kDefaultPerTile[r] ? -1 : h->ts[r].occ[v], v};
    }
    return sh;
}

// table r with tiles of `depth` slices, copied to the device; grid = bps x SMs blocks
int build_role(fr_handle* h, int r, Shape sh, cudaStream_t s = 0) {
    TileSet& t = h->ts[r];
    sh.depth = std::max(sh.depth, kMinDepth);
    {
        const std::vector<int> al = allowed_variants(h, r);
        if (std::find(al.begin(), al.end(), sh.variant) == al.end()) sh.variant = al[0];
    }
    if (sh.bps != -1) sh.bps = std::min(std::max(sh.bps, 1), t.occ[sh.variant]);
    t.shape = sh;
    t.h.clear();
    for (int p = 0; p < h->npairs; ++p) {
        const Pair& P = h->hpairs[p];
        for (int z0 = 0; z0 < P.Z; z0 += sh.depth)
            for (int y0 = 0; y0 < P.Y; y0 += role_tile_y(r, sh.variant))
                for (int x0 = 0; x0 < P.X; x0 += frg::kTileX) t.h.push_back(make_int4(p, x0, y0, z0));
    }
    if (t.h.size() > t.cap) return fail(h, FR_ERR_STATE, "tile table %d overflows (%zu > %zu)", r, t.h.size(), t.cap);
    FR_CUDA(h, cudaMemcpyAsync(t.d, t.h.data(), sizeof(Tile) * t.h.size(), cudaMemcpyHostToDevice, s));
    FR_CUDA(h, cudaStreamSynchronize(s));  // t.h is rewritten by the next build
    t.grid = sh.bps == -1 ? (int)t.h.size()
                          : (int)std::max(1LL, std::min<long long>((long long)sh.bps * h->num_sms, (long long)t.h.size()));
    return FR_OK;
}

int apply_shapes(fr_handle* h, const Shapes& sh, cudaStream_t s = 0) {
    for (int r : active_roles(h)) {
        int rc = build_role(h, r, sh[r], s);
        if (rc != FR_OK) return rc;
    }
    h->graph_valid = false;  // the captured launches carry the old tables
    return FR_OK;
}

// ---- tensor maps of the TMA-staged kernels ----
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, through the runtime (no link against libcuda)
EncodeTiledFn encode_tiled_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    });
    return fn;
}

// A map of a float field of the packed layout: dims[0..rank) innermost first, byte
// strides of dims 1..rank-1, the box copied per request; out-of-volume elements read 0.
int encode_map(fr_handle* h, CUtensorMap* m, const float* base, int rank, const cuuint64_t* dims,
               const cuuint64_t* strides, const cuuint32_t* box) {
    EncodeTiledFn fn = encode_tiled_fn();
    if (!fn) return fail(h, FR_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint32_t ones[5] = {1, 1, 1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, (void*)base, dims, strides, box, ones,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(h, FR_ERR_CUDA, "cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
    return FR_OK;
}

// Every pair's maps (frg::TmapIndex), copied to the device.  Boxes: whole 16-byte chunks
// along x starting at a multiple of 4 floats (the kernels' x coordinates are x0 - 4 or
// x0, x0 a multiple of 32), so every copy starts on a 16-byte boundary.
int encode_tmaps(fr_handle* h) {
    std::vector<CUtensorMap> maps((size_t)h->npairs * frg::TM_COUNT);
    const cuuint64_t fstride = sizeof(float) * (cuuint64_t)h->NT;  // component plane stride
    for (int p = 0; p < h->npairs; ++p) {
        const Pair& P = h->hpairs[p];
        const cuuint64_t Xp = P.Xp, Y = P.Y, Z = P.Z;
        CUtensorMap* m = maps.data() + (size_t)p * frg::TM_COUNT;
        {
            const cuuint64_t dims[4] = {Xp, Y, Z, 3}, strides[3] = {4 * Xp, 4 * Xp * Y, fstride};
            const cuuint32_t box[4] = {40, 10, 1, 3};
            int rc = encode_map(h, m + frg::TM_LAP_PSI, h->psi + P.off, 4, dims, strides, box);
            if (rc != FR_OK) return rc;
        }
        {
            const cuuint64_t dims[3] = {Xp, Y, Z}, strides[2] = {4 * Xp, 4 * Xp * Y};
            const cuuint32_t box[3] = {32, 8, 1};
            int rc = encode_map(h, m + frg::TM_LAP_T, h->T + P.off, 3, dims, strides, box);
            if (rc != FR_OK) return rc;
        }
        if (h->P.solver == FR_SOLVER_REFERENCE) {  // pass A's v, psi_inv, rho (both buffers) and S
            const cuuint64_t d4[4] = {Xp, Y, Z, 3}, s4[3] = {4 * Xp, 4 * Xp * Y, fstride};
            const cuuint64_t d3[3] = {Xp, Y, Z}, s3[2] = {4 * Xp, 4 * Xp * Y};
            const cuuint32_t bv[4] = {40, 12, 1, 3}, bq[4] = {40, 10, 1, 3}, b3[3] = {40, 10, 1};
            for (int k = 0; k < 2; ++k) {
                int rc = encode_map(h, m + frg::TM_PA_V0 + k, h->v[k] + P.off, 4, d4, s4, bv);
                if (rc == FR_OK) rc = encode_map(h, m + frg::TM_PA_Q0 + k, h->pinv[k] + P.off, 4, d4, s4, bq);
                if (rc == FR_OK) rc = encode_map(h, m + frg::TM_PA_R0 + k, h->rho[k] + P.off, 3, d3, s3, b3);
                if (rc != FR_OK) return rc;
            }
            int rc = encode_map(h, m + frg::TM_PA_S, h->S + P.off, 3, d3, s3, b3);
            if (rc != FR_OK) return rc;
        }
        {  // the gathered field of the update kernel: v (both buffers) or the momentum
            const cuuint64_t d4[4] = {Xp, Y, Z, 3}, s4[3] = {4 * Xp, 4 * Xp * Y, fstride};
            const cuuint32_t bg[4] = {frg::kGBX, frg::kGBY, frg::kGBZ, 3};
            const int nb = h->P.solver == FR_SOLVER_REFERENCE ? 2 : 1;
            for (int k = 0; k < nb; ++k) {
                int rc = encode_map(h, m + (nb == 2 ? frg::TM_PB_V0 + k : frg::TM_SB_M), h->v[k] + P.off, 4, d4, s4,
                                    bg);
                if (rc != FR_OK) return rc;
            }
        }
        if (h->P.solver == FR_SOLVER_SOBOLEV) {
            int wx = 0, rows = 0;
            frg::sob_smooth_box(h->P.smooth_width / 2, &wx, &rows);
            const cuuint64_t dims[4] = {Xp, Y, Z, 3}, strides[3] = {4 * Xp, 4 * Xp * Y, fstride};
            const cuuint32_t box[4] = {(cuuint32_t)wx, (cuuint32_t)rows, 1, 3};
            int rc = encode_map(h, m + frg::TM_SOB_G, h->grad + P.off, 4, dims, strides, box);
            if (rc != FR_OK) return rc;
        }
    }
    FR_CUDA(h, cudaMemcpy(h->tmaps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice));
    return FR_OK;
}

// (Re)build the packed cohort for the given pair sizes.
int setup_cohort(fr_handle* h, const fr_pair* pairs, int n) {
    std::vector<std::array<int, 3>> dims(n);
    for (int p = 0; p < n; ++p) {
        for (int c = 0; c < 3; ++c) {
            if (pairs[p].dims[c] < 4)
                return fail(h, FR_ERR_INVALID_ARG, "pair %d dims[%d] = %d < 4 (the solver needs an interior)", p, c,
                            pairs[p].dims[c]);
            dims[p][c] = pairs[p].dims[c];
        }
        const long long Xp = (dims[p][0] + 3) / 4 * 4, Np = Xp * dims[p][1] * dims[p][2];
        if (!frg::fits_index32(Xp, dims[p][1], dims[p][2]))
            return fail(h, FR_ERR_INVALID_ARG,
                        "pair %d is too large (%lld padded voxels: the kernels' 32-bit offsets need "
                        "N + 2 X Y + 2 X + 2 <= 2^31-1)", p, Np);
    }
    const int want_trace = std::max(h->P.max_iter, 1);
    if (h->block && dims == h->dims && h->trace_cap >= want_trace) return FR_OK;
    release(h);

    h->dims = dims;
    h->npairs = n;
    h->hpairs.assign(n, Pair{});
    h->htiles.clear();
    long long off = 0;
    for (int p = 0; p < n; ++p) {
        Pair& P = h->hpairs[p];
        P.X = dims[p][0];
        P.Y = dims[p][1];
        P.Z = dims[p][2];
        P.Xp = (P.X + 3) / 4 * 4;  // rows on 16-byte boundaries
        P.N = (long long)P.Xp * P.Y * P.Z;
        P.off = off;
        P.w_reg = h->P.w_reg;
        off += (long long)align_up((size_t)P.N, 32);
        for (int z0 = 0; z0 < P.Z; z0 += frg::kTileZ)  // the I/O kernels' table
            for (int y0 = 0; y0 < P.Y; y0 += frg::kTileY)
                for (int x0 = 0; x0 < P.X; x0 += frg::kTileX) h->htiles.push_back(make_int4(p, x0, y0, z0));
    }
    h->NT = std::max(off, 32LL);
    const long long NT = h->NT;
    const int ntiles = (int)h->htiles.size();
    h->trace_cap = want_trace;

    // carve one allocation
    struct Slot {
        void** ptr;
        size_t bytes;
    };
    std::vector<Slot> slots;
    auto add = [&](void** p, size_t bytes) { slots.push_back({p, bytes}); };
    add((void**)&h->d_pairs, sizeof(Pair) * n);
    add((void**)&h->d_tiles, sizeof(Tile) * ntiles);
    // the solver kernels' tables, each with room for the shallowest and lowest tiles
    size_t cap = 0;
    const int min_tile_y = std::min(frg::kTileY, frg::kPassBTileY);
    for (const Pair& P : h->hpairs)
        cap += (size_t)((P.X + frg::kTileX - 1) / frg::kTileX) * ((P.Y + min_tile_y - 1) / min_tile_y) *
               ((P.Z + kMinDepth - 1) / kMinDepth);
    for (int r : active_roles(h)) {
        h->ts[r].cap = cap;
        add((void**)&h->ts[r].d, sizeof(Tile) * cap);
    }
    add((void**)&h->d_io, sizeof(frg::PairIO) * n);
    add((void**)&h->S, sizeof(float) * NT);
    add((void**)&h->T, sizeof(float) * NT);
    add((void**)&h->labS, sizeof(int16_t) * NT);
    add((void**)&h->labT, sizeof(int16_t) * NT);
    add((void**)&h->psi, sizeof(float) * 3 * NT);
    add((void**)&h->v[0], sizeof(float) * 3 * NT);
    add((void**)&h->v[1], sizeof(float) * 3 * NT);
    if (h->P.solver == FR_SOLVER_REFERENCE) {
        add((void**)&h->rho[0], sizeof(float) * NT);
        add((void**)&h->rho[1], sizeof(float) * NT);
        add((void**)&h->pinv[0], sizeof(float) * 3 * NT);
        add((void**)&h->pinv[1], sizeof(float) * 3 * NT);
        add((void**)&h->LT, sizeof(float4) * NT);
    } else {
        h->rho[0] = h->rho[1] = h->pinv[0] = h->pinv[1] = nullptr;
        h->LT = nullptr;
        add((void**)&h->grad, sizeof(float) * 3 * NT);
        add((void**)&h->sob_energy, sizeof(double) * (size_t)n * want_trace);
    }
    add((void**)&h->stop, sizeof(int) * n);
    add((void**)&h->keys, sizeof(unsigned long long) * n);
    add((void**)&h->trace, sizeof(unsigned long long) * (size_t)n * want_trace);
    add((void**)&h->counter, sizeof(unsigned int) * 4);
    add((void**)&h->dev_err, sizeof(unsigned int));
    add((void**)&h->tmaps, sizeof(CUtensorMap) * (size_t)n * frg::TM_COUNT);
    add((void**)&h->tile_partials, sizeof(double) * 2 * ntiles);
    add((void**)&h->pair_tiles, sizeof(int) * (n + 1));
    add((void**)&h->tile_folds, sizeof(long long) * ntiles);
    add((void**)&h->dice, sizeof(unsigned long long) * (size_t)n * (2 * 256 + 1));
    add((void**)&h->pair_energy, sizeof(double) * 2 * n);
    add((void**)&h->pair_folds, sizeof(long long) * n);
    size_t total = 0;
    for (auto& s : slots) total = align_up(total, 256) + s.bytes;
    total = align_up(total, 256);
    cudaError_t e = cudaMalloc((void**)&h->block, total);
    if (e != cudaSuccess) {
        h->block = nullptr;
        cudaGetLastError();
        h->dims.clear();
        return fail(h, FR_ERR_ALLOC, "cudaMalloc of %zu bytes for %d pair(s) failed: %s", total, n,
                    cudaGetErrorString(e));
    }
    h->block_bytes = total;
    size_t at = 0;
    for (auto& s : slots) {
        at = align_up(at, 256);
        *s.ptr = h->block + at;
        at += s.bytes;
    }
    // everything starts at zero: L's boundary shell, counters, partials
    FR_CUDA(h, cudaMemset(h->block, 0, total));
    FR_CUDA(h, cudaMemcpy(h->d_pairs, h->hpairs.data(), sizeof(Pair) * n, cudaMemcpyHostToDevice));
    FR_CUDA(h, cudaMemcpy(h->d_tiles, h->htiles.data(), sizeof(Tile) * ntiles, cudaMemcpyHostToDevice));
    {
        std::vector<int> first(n + 1, ntiles);
        for (int t = ntiles - 1; t >= 0; --t) first[h->htiles[t].x] = t;
        for (int p = n - 1; p >= 0; --p) first[p] = std::min(first[p], first[p + 1]);
        FR_CUDA(h, cudaMemcpy(h->pair_tiles, first.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    }
    if (h->P.solver == FR_SOLVER_REFERENCE) {
        FR_CUDA(h, cudaFuncSetAttribute((const void*)frg::ref_pass_a_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)frg::ref_pass_a_smem_bytes()));
        FR_CUDA(h, cudaFuncSetAttribute((const void*)frg::ref_pass_a_tma_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)frg::ref_pass_a_tma_smem_bytes()));
    }
    FR_CUDA(h, cudaFuncSetAttribute(role_fn(h, h->P.solver == FR_SOLVER_REFERENCE ? R_PB : R_SB, 1),
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)frg::gather_staged_smem_bytes()));
    h->tma_ok = encode_tmaps(h) == FR_OK;
    if (!h->tma_ok && h->P.staging == 2) {
        const std::string why = h->err;
        release(h);
        return fail(h, FR_ERR_CUDA, "STAGING=2 asks for TMA staging, but the tensor maps could not be made (%s)",
                    why.c_str());
    }
    h->err.clear();  // a cohort whose maps cannot be encoded runs the cp.async variants
    for (int r : active_roles(h))
        for (int v = 0; v < (has_tma_variant(r) ? 2 : 1); ++v) {
            int occ = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, role_fn(h, r, v), role_threads(r, v),
                                                              role_smem(r, v)) !=
                    cudaSuccess ||
                occ < 1)
                occ = 1;
            h->ts[r].occ[v] = occ;
        }
    h->tuned = false;
    {
        int rc = apply_shapes(h, default_shapes(h));
        if (rc != FR_OK) return rc;
    }
    h->grid_io = occupancy_grid(h, (const void*)frg::finalize_kernel, ntiles);
    return FR_OK;
}

frg::RefIterArgs ref_args(fr_handle* h, int iter, float t) {
    frg::RefIterArgs a{};
    a.pairs = h->d_pairs;
    a.tiles_l = h->ts[R_LAP].d;
    a.ntiles_l = (int)h->ts[R_LAP].h.size();
    a.depth_l = h->ts[R_LAP].shape.depth;
    a.tiles_a = h->ts[R_PA].d;
    a.ntiles_a = (int)h->ts[R_PA].h.size();
    a.depth_a = h->ts[R_PA].shape.depth;
    a.tiles_b = h->ts[R_PB].d;
    a.ntiles_b = (int)h->ts[R_PB].h.size();
    a.depth_b = h->ts[R_PB].shape.depth;
    a.npairs = h->npairs;
    a.NT = h->NT;
    a.S = h->S;
    a.T = h->T;
    const int src = (iter - 1) & 1, dst = iter & 1;
    a.rho = h->rho[src];
    a.v = h->v[src];
    a.pinv = h->pinv[src];
    a.rho_n = h->rho[dst];
    a.v_n = h->v[dst];
    a.pinv_n = h->pinv[dst];
    a.psi = h->psi;
    a.LT = h->LT;
    const fr_params& P = h->P;
    // solver.cu:198-199, evaluated once per iteration on the host in float
    const float m1 = P.p + 1.f;
    a.alpha = P.alpha;
    a.f1 = m1 / t;
    a.m2 = (P.C * powf(P.p, 2.f)) * powf(t, P.p - 2.f);
    a.tau = P.tau;
    a.w_reg = P.w_reg;
    a.max_update_norm = P.max_update_norm;
    a.iter = iter;
    a.first_iter = iter == 1;
    a.stop = h->stop;
    a.keys = h->keys;
    a.trace = h->trace;
    a.counter = h->counter;
    a.tmaps = h->tmaps;
    a.err = h->dev_err;
    return a;
}

int launch_ref_iter(fr_handle* h, int iter, float t, cudaStream_t s, cudaEvent_t* ev) {
    frg::RefIterArgs a = ref_args(h, iter, t);
    if (ev) cudaEventRecord(ev[0], s);
    if (h->ts[R_LAP].shape.variant)
        frg::ref_laplacian_tma_kernel<<<h->ts[R_LAP].grid, 256, frg::ref_laplacian_tma_smem_bytes(), s>>>(a);
    else
        frg::ref_laplacian_kernel<<<h->ts[R_LAP].grid, 256, frg::ref_laplacian_smem_bytes(), s>>>(a);
    if (ev) cudaEventRecord(ev[1], s);
    if (h->ts[R_PA].shape.variant)
        frg::ref_pass_a_tma_kernel<<<h->ts[R_PA].grid, 256, frg::ref_pass_a_tma_smem_bytes(), s>>>(a);
    else
        frg::ref_pass_a_kernel<<<h->ts[R_PA].grid, 256, frg::ref_pass_a_smem_bytes(), s>>>(a);
    if (ev) cudaEventRecord(ev[2], s);
    if (h->ts[R_PB].shape.variant)
        frg::ref_pass_b_staged_kernel<<<h->ts[R_PB].grid, 256, frg::gather_staged_smem_bytes(), s>>>(a);
    else
        frg::ref_pass_b_kernel<<<h->ts[R_PB].grid, frg::kPassBThreads, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[3], s);
    FR_LAUNCHED(h);
    return FR_OK;
}

// kernels launched per iteration (three in either solver)
int kernels_per_iter(const fr_handle*) { return 3; }

frg::SobIterArgs sob_args(fr_handle* h, int iter) {
    frg::SobIterArgs a{};
    a.pairs = h->d_pairs;
    a.tiles_g = h->ts[R_SG].d;
    a.ntiles_g = (int)h->ts[R_SG].h.size();
    a.depth_g = h->ts[R_SG].shape.depth;
    a.tiles_s = h->ts[R_SS].d;
    a.ntiles_s = (int)h->ts[R_SS].h.size();
    a.depth_s = h->ts[R_SS].shape.depth;
    a.tiles_b = h->ts[R_SB].d;
    a.ntiles_b = (int)h->ts[R_SB].h.size();
    a.depth_b = h->ts[R_SB].shape.depth;
    a.npairs = h->npairs;
    a.NT = h->NT;
    a.S = h->S;
    a.T = h->T;
    a.phi = h->psi;
    a.m = h->v[0];
    a.g = h->grad;
    a.damping = h->P.damping;
    a.step = h->P.step;
    a.lambda = h->P.w_reg;
    frg::gaussian_taps(h->P.smooth_sigma, h->P.smooth_width, a.taps);
    a.radius = h->P.smooth_width / 2;
    a.max_update_norm = h->P.max_update_norm;
    a.iter = iter;
    a.stop = h->stop;
    a.keys = h->keys;
    a.trace = h->trace;
    a.energy = h->sob_energy;
    a.counter = h->counter;
    a.tmaps = h->tmaps;
    a.err = h->dev_err;
    return a;
}

int launch_iter(fr_handle* h, int iter, float t, cudaStream_t s, cudaEvent_t* ev = nullptr) {
    if (h->P.solver == FR_SOLVER_REFERENCE) return launch_ref_iter(h, iter, t, s, ev);
    const frg::SobIterArgs a = sob_args(h, iter);
    const int grids[3] = {h->ts[R_SG].grid, h->ts[R_SS].grid, h->ts[R_SB].grid};
    const int variants[3] = {h->ts[R_SG].shape.variant, h->ts[R_SS].shape.variant, h->ts[R_SB].shape.variant};
    cudaError_t e = frg::launch_sob_iter(a, grids, variants, s, ev);
    if (e != cudaSuccess) return fail(h, FR_ERR_CUDA, "sobolev launch failed: %s", cudaGetErrorString(e));
    return FR_OK;
}

frg::IoArgs io_args(fr_handle* h) {
    frg::IoArgs a{};
    a.pairs = h->d_pairs;
    a.tiles = h->d_tiles;
    a.ntiles = (int)h->htiles.size();
    a.npairs = h->npairs;
    a.NT = h->NT;
    a.io = h->d_io;
    a.S = h->S;
    a.T = h->T;
    a.labS = h->labS;
    a.labT = h->labT;
    a.rho0 = h->rho[0];
    a.rho1 = h->rho[1];
    a.v0 = h->v[0];
    a.v1 = h->v[1];
    a.psi = h->psi;
    a.pinv0 = h->pinv[0];
    a.pinv1 = h->pinv[1];
    a.LT = h->LT;
    a.rho_init = h->P.rho_0;
    a.keep_state = h->P.keep_state && h->have_state;
    a.sobolev = h->P.solver == FR_SOLVER_SOBOLEV;
    a.stop = h->stop;
    a.max_iter = h->last_iter;
    a.no_labels = h->P.no_labels;
    a.tile_partials = h->tile_partials;
    a.pair_tiles = h->pair_tiles;
    a.tile_folds = h->tile_folds;
    a.dice = h->dice;
    a.pair_energy = h->pair_energy;
    a.pair_folds = h->pair_folds;
    a.counter = h->counter + 1;
    a.write_outputs = 1;
    return a;
}

// Move each pair's final state into buffer 0 so that a KEEP_STATE call starts from it.
int normalise_parity(fr_handle* h) {
    if (h->P.solver != FR_SOLVER_REFERENCE || !h->have_state) return FR_OK;
    std::vector<int> stop(h->npairs);
    FR_CUDA(h, cudaDeviceSynchronize());
    FR_CUDA(h, cudaMemcpy(stop.data(), h->stop, sizeof(int) * h->npairs, cudaMemcpyDeviceToHost));
    for (int p = 0; p < h->npairs; ++p) {
        int done = stop[p] ? stop[p] : h->last_iter;
        if (!(done & 1)) continue;
        const Pair& P = h->hpairs[p];
        FR_CUDA(h, cudaMemcpy(h->rho[0] + P.off, h->rho[1] + P.off, sizeof(float) * P.N, cudaMemcpyDeviceToDevice));
        for (int c = 0; c < 3; ++c) {
            FR_CUDA(h, cudaMemcpy(h->v[0] + c * h->NT + P.off, h->v[1] + c * h->NT + P.off, sizeof(float) * P.N,
                                  cudaMemcpyDeviceToDevice));
            FR_CUDA(h, cudaMemcpy(h->pinv[0] + c * h->NT + P.off, h->pinv[1] + c * h->NT + P.off,
                                  sizeof(float) * P.N, cudaMemcpyDeviceToDevice));
        }
    }
    return FR_OK;
}

int host_stats(fr_handle* h);

int verbose_energy(fr_handle* h, int iter, cudaStream_t s, double* energy) {
    frg::IoArgs a = io_args(h);
    a.write_outputs = 0;
    a.max_iter = iter - 1;  // state after iter-1 iterations
    if (h->P.solver == FR_SOLVER_SOBOLEV) a.sobolev = 1;
    FR_CUDA(h, cudaMemsetAsync(h->dice, 0, sizeof(unsigned long long) * h->npairs * (2 * 256 + 1), s));
    frg::finalize_kernel<<<h->grid_io, 256, 0, s>>>(a);
    FR_LAUNCHED(h);
    std::vector<double> e(2 * h->npairs);
    FR_CUDA(h, cudaMemcpyAsync(e.data(), h->pair_energy, sizeof(double) * 2 * h->npairs, cudaMemcpyDeviceToHost, s));
    FR_CUDA(h, cudaStreamSynchronize(s));
    for (int p = 0; p < h->npairs; ++p) {
        const double w = h->hpairs[p].w_reg;
        double val = e[2 * p] + w * e[2 * p + 1];
        printf("data energy + w_reg * reg energy = %g + %g * %g = %g\n", e[2 * p], w, e[2 * p + 1],
               val);
        if (p == 0) *energy = val;
    }
    return FR_OK;
}

int run_registration(fr_handle* h, cudaStream_t s) {
    const fr_params& P = h->P;
    std::vector<float> ts = t_schedule(P);
    h->last_iter = P.max_iter;
    if (P.verbosity == 0) {
        if (P.max_iter > 0) {
            if (!h->graph_valid) {
                if (!h->cap_stream) FR_CUDA(h, cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking));
                FR_CUDA(h, cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
                int rc = FR_OK;
                for (int it = 1; it <= P.max_iter && rc == FR_OK; ++it) rc = launch_iter(h, it, ts[it - 1], h->cap_stream);
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamEndCapture(h->cap_stream, &g);
                if (rc != FR_OK) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                if (e != cudaSuccess) return fail(h, FR_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
                if (h->graph) cudaGraphExecDestroy(h->graph);
                h->graph = nullptr;
                e = cudaGraphInstantiate(&h->graph, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return fail(h, FR_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
                h->graph_valid = true;
            }
            FR_CUDA(h, cudaGraphLaunch(h->graph, s));
        }
        return FR_OK;
    }
    // verbose: host-driven loop with the reference's prints (solver.cu:329-433)
    std::vector<int> stop(h->npairs, 0);
    for (int iter = 1; iter <= P.max_iter; ++iter) {
        if (iter == 1 || iter % 100 == 0) printf("iter. no. %d\n", iter);
        bool report = (P.verbosity == 1 && (iter == 1 || iter % 100 == 0 || iter == P.max_iter)) || P.verbosity == 2;
        if (report) {
            double e = 0.0;
            int rc = verbose_energy(h, iter, s, &e);
            if (rc != FR_OK) return rc;
            if (std::isnan(e)) {
                h->last_iter = iter - 1;
                return fail(h, FR_ERR_NUMERIC, "energy is NaN at iteration %d", iter);
            }
        }
        int rc = launch_iter(h, iter, ts[iter - 1], s);
        if (rc != FR_OK) return rc;
        std::vector<unsigned long long> k(h->npairs);
        FR_CUDA(h, cudaMemcpyAsync(k.data(), h->trace + (size_t)(iter - 1) * h->npairs,
                                   sizeof(unsigned long long) * h->npairs, cudaMemcpyDeviceToHost, s));
        FR_CUDA(h, cudaMemcpyAsync(stop.data(), h->stop, sizeof(int) * h->npairs, cudaMemcpyDeviceToHost, s));
        FR_CUDA(h, cudaStreamSynchronize(s));
        if (report) {
            float mx;
            long long ip;
            decode_key(k[0], &mx, &ip);
            const Pair& P0 = h->hpairs[0];
            const long long idx = user_index(P0, ip);
            long long zz = idx / ((long long)P0.X * P0.Y);
            long long yy = (idx - zz * P0.X * P0.Y) / P0.X;
            long long xx = idx - P0.X * (yy + (long long)P0.Y * zz);
            printf("max. update norm %g at voxel (%lld, %lld, %lld)\n", (double)mx, xx, yy, zz);
        }
        bool all_stopped = true;
        for (int p = 0; p < h->npairs; ++p) all_stopped = all_stopped && stop[p] != 0;
        if (all_stopped) {
            printf("SOLVER CONVERGED AFTER %d ITERATIONS\n", iter);
            h->last_iter = iter;
            return FR_OK;
        }
        if (iter == P.max_iter) printf("SOLVER REACHED MAX. NO. OF ITERATIONS WITHOUT CONVERGING\n");
        fflush(stdout);
    }
    return FR_OK;
}

// ---- autotuner ----
// For each solver kernel, a few tile depths and blocks-per-SM counts are timed on the
// freshly packed cohort (identity state, iteration 1), the kernel launched alone; the
// fastest shape is kept.  The choice is cached per size class (solver, SM count,
// smoothing width and the multiset of pair sizes) for the life of the process.  A tile
// shape changes which block computes a voxel, never how, so results do not depend on it.
std::string size_class(const fr_handle* h) {
    std::ostringstream k;
    k << h->P.solver << '/' << h->device << '/' << h->num_sms << '/'
      << (h->P.solver == FR_SOLVER_SOBOLEV ? h->P.smooth_width : 0) << '/' << h->P.staging;
    std::vector<std::array<int, 3>> d = h->dims;
    std::sort(d.begin(), d.end());
    for (const auto& x : d) k << '/' << x[0] << 'x' << x[1] << 'x' << x[2];
    return k.str();
}

std::mutex g_tune_mu;
std::map<std::string, Shapes> g_tuned;

int launch_role(fr_handle* h, int r, int iter, float t, cudaStream_t s) {
    frg::RefIterArgs ra{};
    frg::SobIterArgs sa{};
    void* args[1];
    // no pair converges while shapes are timed (a stopped pair's tiles would be skipped)
    if (r == R_LAP || r == R_PA || r == R_PB) {
        ra = ref_args(h, iter, t);
        ra.max_update_norm = -INFINITY;
        args[0] = &ra;
    } else {
        sa = sob_args(h, iter);
        sa.max_update_norm = -INFINITY;
        args[0] = &sa;
    }
    const int v = h->ts[r].shape.variant;
    FR_CUDA(h, cudaLaunchKernel(role_fn(h, r, v), dim3(h->ts[r].grid), dim3(role_threads(r, v)), args,
                                role_smem(r, v), s));
    return FR_OK;
}

int autotune(fr_handle* h, cudaStream_t s) {
    const std::string key = size_class(h);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            int rc = apply_shapes(h, it->second, s);
            if (rc == FR_OK) h->tuned = true;
            return rc;
        }
    }
    // a state to time on: the packed cohort of the current registration after a few
    // iterations (an even number, so that the double-buffered fields are back in buffer
    // 0), where the velocity or momentum that the update kernels gather is no longer zero
    // and the gathers leave the grid points; shapes timed at the identity state chose a
    // sobolev update 7% slower than the best
    FR_CUDA(h, cudaMemsetAsync(h->stop, 0, sizeof(int) * h->npairs, s));
    frg::IoArgs io = io_args(h);
    io.keep_state = 0;
    frg::pack_init_kernel<<<h->grid_io, 256, 0, s>>>(io);
    FR_LAUNCHED(h);
    const std::vector<float> ts = t_schedule(h->P);
    const int warm = std::min(kTuneWarmIters, (h->trace_cap - 1) / 2 * 2);  // the trace holds iteration warm + 1
    for (int it = 1; it <= warm; ++it) {
        int rc = launch_iter(h, it, ts[it - 1], s);
        if (rc != FR_OK) return rc;
    }
    const int iter = warm + 1;
    const float t = iter <= (int)ts.size() ? ts[iter - 1] : h->P.alpha;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return fail(h, FR_ERR_CUDA, "autotune: cudaEventCreate failed");
    }
    Shapes best = default_shapes(h);
    // tile depths: a fixed ladder, plus ceil(Zmax / k), which cut the tallest pair's columns
    // into k tiles of (nearly) equal depth, so that the tile count can match the GPU's
    // resident blocks more closely than the ladder's steps allow
    std::vector<int> depths = {1, 2, 4, 8, 12, 16, 24, 32, 48, 64, 96};
    {
        int zmax = 1;
        for (const Pair& P : h->hpairs) zmax = std::max(zmax, P.Z);
        for (int k = 1; k <= 32; ++k) depths.push_back((zmax + k - 1) / k);
        std::sort(depths.begin(), depths.end());
        depths.erase(std::unique(depths.begin(), depths.end()), depths.end());
    }
    int rc = FR_OK;
    for (int r : active_roles(h)) {
        std::vector<Shape> cand;
        for (int v : allowed_variants(h, r)) {
            const int occ = h->ts[r].occ[v];
            std::vector<int> bps = {occ};
            if (occ > 1) bps.push_back(occ - 1);
            if (occ / 2 >= 1 && occ / 2 < occ - 1) bps.push_back(occ / 2);
            bps.push_back(-1);  // one block per tile
            for (int depth : depths)
                for (int b : bps) cand.push_back(Shape{depth, b, v});
        }
        // two passes over the candidates, each candidate's faster time kept (less noise)
        std::vector<float> best_of(cand.size(), 1e30f);
        for (int pass = 0; pass < 2 && rc == FR_OK; ++pass) {
            for (size_t ci = 0; ci < cand.size() && rc == FR_OK; ++ci) {
                rc = build_role(h, r, cand[ci], s);
                if (rc != FR_OK) break;
                if (cudaMemsetAsync(h->stop, 0, sizeof(int) * h->npairs, s) != cudaSuccess) {
                    rc = fail(h, FR_ERR_CUDA, "autotune: memset failed");
                    break;
                }
                rc = launch_role(h, r, iter, t, s);  // warm-up
                if (rc == FR_OK) cudaEventRecord(e0, s);
                for (int k = 0; k < 3 && rc == FR_OK; ++k) rc = launch_role(h, r, iter, t, s);
                if (rc != FR_OK) break;
                cudaEventRecord(e1, s);
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    rc = fail(h, FR_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                best_of[ci] = std::min(best_of[ci], ms);
            }
        }
        if (rc != FR_OK) break;
        size_t win = 0;
        for (size_t ci = 1; ci < cand.size(); ++ci)
            if (best_of[ci] < best_of[win]) win = ci;
        rc = build_role(h, r, cand[win], s);
        if (rc != FR_OK) break;
        best[r] = h->ts[r].shape;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FR_OK) return rc;
    rc = check_device_error(h);
    if (rc != FR_OK) return rc;
    h->graph_valid = false;
    h->tuned = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best;
    return FR_OK;
}

int begin(fr_handle* h, const fr_pair* pairs, int n, cudaStream_t s) {
    if (!pairs || n < 1) return fail(h, FR_ERR_INVALID_ARG, "need at least one pair");
    for (int p = 0; p < n; ++p)
        if (!pairs[p].img_T || !pairs[p].lab_T || !pairs[p].img_S || !pairs[p].lab_S)
            return fail(h, FR_ERR_INVALID_ARG, "pair %d has a NULL buffer", p);
    bool same = h->block && (int)h->dims.size() == n;
    for (int p = 0; same && p < n; ++p)
        for (int c = 0; c < 3; ++c) same = same && h->dims[p][c] == pairs[p].dims[c];
    if (h->P.keep_state && same && h->have_state) {
        int rc = normalise_parity(h);
        if (rc != FR_OK) return rc;
    }
    if (!h->pair_w_reg.empty() && (int)h->pair_w_reg.size() != n)
        return fail(h, FR_ERR_INVALID_ARG, "fr_set_pair_w_reg gave %zu weights for a cohort of %d pairs",
                    h->pair_w_reg.size(), n);
    int rc = setup_cohort(h, pairs, n);
    if (rc != FR_OK) return rc;
    if (!same) h->have_state = false;
    {  // each pair's regularisation weight (read by the kernels from the pair table)
        bool changed = false;
        for (int p = 0; p < n; ++p) {
            const float w = h->pair_w_reg.empty() ? h->P.w_reg : h->pair_w_reg[p];
            if (h->hpairs[p].w_reg != w) {
                h->hpairs[p].w_reg = w;
                changed = true;
            }
        }
        if (changed) FR_CUDA(h, cudaMemcpyAsync(h->d_pairs, h->hpairs.data(), sizeof(Pair) * n, cudaMemcpyHostToDevice, s));
    }
    h->io.assign(pairs, pairs + n);
    std::vector<frg::PairIO> io(n);
    for (int p = 0; p < n; ++p) io[p] = frg::PairIO{pairs[p].img_T, pairs[p].lab_T, pairs[p].img_S, pairs[p].lab_S};
    FR_CUDA(h, cudaMemcpyAsync(h->d_io, io.data(), sizeof(frg::PairIO) * n, cudaMemcpyHostToDevice, s));
    if (h->P.autotune && !h->tuned && !(h->P.keep_state && h->have_state)) {
        rc = autotune(h, s);  // leaves the state to the initialisation below
        if (rc != FR_OK) return rc;
    }
    FR_CUDA(h, cudaMemsetAsync(h->stop, 0, sizeof(int) * n, s));
    FR_CUDA(h, cudaMemsetAsync(h->dev_err, 0, sizeof(unsigned int), s));
    FR_CUDA(h, cudaMemsetAsync(h->keys, 0, sizeof(unsigned long long) * n, s));
    FR_CUDA(h, cudaMemsetAsync(h->trace, 0, sizeof(unsigned long long) * n * (size_t)h->trace_cap, s));
    if (h->sob_energy)
        FR_CUDA(h, cudaMemsetAsync(h->sob_energy, 0, sizeof(double) * n * (size_t)h->trace_cap, s));
    frg::IoArgs a = io_args(h);
    frg::pack_init_kernel<<<h->grid_io, 256, 0, s>>>(a);
    FR_LAUNCHED(h);
    h->have_state = true;
    h->finished = false;
    h->stats_ready = false;
    h->last_iter = 0;
    h->last_stream = s;
    return FR_OK;
}

int finish(fr_handle* h, cudaStream_t s) {
    FR_CUDA(h, cudaMemsetAsync(h->dice, 0, sizeof(unsigned long long) * h->npairs * (2 * 256 + 1), s));
    frg::IoArgs a = io_args(h);
    frg::finalize_kernel<<<h->grid_io, 256, 0, s>>>(a);
    FR_LAUNCHED(h);
    h->finished = true;
    h->last_stream = s;
    return FR_OK;
}

int host_stats(fr_handle* h) {
    if (h->stats_ready) return FR_OK;
    const int n = h->npairs;
    FR_CUDA(h, cudaStreamSynchronize(h->last_stream));
    std::vector<int> stop(n);
    std::vector<double> energy(2 * n);
    std::vector<long long> folds(n);
    std::vector<unsigned long long> dice((size_t)n * (2 * 256 + 1));
    std::vector<unsigned long long> trace((size_t)n * h->trace_cap);
    {
        int rc = check_device_error(h);
        if (rc != FR_OK) return rc;
    }
    FR_CUDA(h, cudaMemcpy(stop.data(), h->stop, sizeof(int) * n, cudaMemcpyDeviceToHost));
    FR_CUDA(h, cudaMemcpy(energy.data(), h->pair_energy, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    FR_CUDA(h, cudaMemcpy(folds.data(), h->pair_folds, sizeof(long long) * n, cudaMemcpyDeviceToHost));
    FR_CUDA(h, cudaMemcpy(dice.data(), h->dice, sizeof(unsigned long long) * dice.size(), cudaMemcpyDeviceToHost));
    FR_CUDA(h, cudaMemcpy(trace.data(), h->trace, sizeof(unsigned long long) * trace.size(), cudaMemcpyDeviceToHost));
    h->stats.assign(n, fr_stats{});
    for (int p = 0; p < n; ++p) {
        fr_stats& st = h->stats[p];
        st.converged = stop[p] != 0;
        st.iterations = stop[p] ? stop[p] : h->last_iter;
        if (st.iterations > 0) {
            long long ip;
            decode_key(trace[(size_t)(st.iterations - 1) * n + p], &st.last_max_update_norm, &ip);
            st.last_max_update_voxel = (int64_t)user_index(h->hpairs[p], ip);
        }
        st.e_data = energy[2 * p];
        st.e_reg = energy[2 * p + 1];
        st.energy = st.e_data + (double)h->hpairs[p].w_reg * st.e_reg;
        st.folds = folds[p];
        st.no_labels = h->P.no_labels;
        const unsigned long long* dp = dice.data() + (size_t)p * (2 * 256 + 1);
        double num = 0.0, den = 0.0;
        for (int l = 0; l < FR_MAX_LABELS; ++l) {
            st.dice_inter[l] = (int64_t)dp[l];
            st.dice_count[l] = (int64_t)dp[256 + l];
            st.dice[l] = dp[256 + l] ? 2.0 * (double)dp[l] / (double)dp[256 + l] : NAN;
            if (l >= 1 && l < h->P.no_labels) {
                num += (double)dp[l];
                den += (double)dp[256 + l];
            }
        }
        st.dice_all = den > 0 ? 2.0 * num / den : NAN;
        st.dice_out_of_range = (int64_t)dp[2 * 256];
    }
    h->stats_ready = true;
    return FR_OK;
}

// params.ini: KEY=VALUE lines, '#' comments (boost::program_options::parse_config_file
// syntax as used by demo.cpp:144-149)
int set_key(fr_params* p, const std::string& key, const std::string& val, std::string* why) {
    auto as_int = [&](int* dst) -> bool {
        char* end = nullptr;
        long v = strtol(val.c_str(), &end, 10);
        if (!end || *end != '\0' || val.empty()) return false;
        *dst = (int)v;
        return true;
    };
    auto as_float = [&](float* dst) -> bool {
        char* end = nullptr;
        float v = strtof(val.c_str(), &end);
        if (!end || *end != '\0' || val.empty()) return false;
        *dst = v;
        return true;
    };
    bool ok = true;
    if (key == "VOL_DIMS_X") ok = as_int(&p->volume_dims[0]);
    else if (key == "VOL_DIMS_Y") ok = as_int(&p->volume_dims[1]);
    else if (key == "VOL_DIMS_Z") ok = as_int(&p->volume_dims[2]);
    else if (key == "VOL_SIZE_X") ok = as_float(&p->volume_size[0]);
    else if (key == "VOL_SIZE_Y") ok = as_float(&p->volume_size[1]);
    else if (key == "VOL_SIZE_Z") ok = as_float(&p->volume_size[2]);
    else if (key == "NO_LABELS") ok = as_int(&p->no_labels);
    else if (key == "MAX_ITER") ok = as_int(&p->max_iter);
    else if (key == "MAX_UPDATE_NORM") ok = as_float(&p->max_update_norm);
    else if (key == "RHO_0") ok = as_float(&p->rho_0);
    else if (key == "RESET_ITER") ok = as_int(&p->reset_iter);
    else if (key == "TAU") ok = as_float(&p->tau);
    else if (key == "ALPHA") ok = as_float(&p->alpha);
    else if (key == "W_REG") ok = as_float(&p->w_reg);
    else if (key == "p") ok = as_float(&p->p);
    else if (key == "C") ok = as_float(&p->C);
    else if (key == "VERBOSITY") ok = as_int(&p->verbosity);
    else if (key == "SOLVER") {
        if (val == "reference") p->solver = FR_SOLVER_REFERENCE;
        else if (val == "sobolev") p->solver = FR_SOLVER_SOBOLEV;
        else ok = false;
    } else if (key == "SMOOTH_SIGMA") ok = as_float(&p->smooth_sigma);
    else if (key == "SMOOTH_WIDTH") ok = as_int(&p->smooth_width);
    else if (key == "DAMPING") ok = as_float(&p->damping);
    else if (key == "STEP") ok = as_float(&p->step);
    else if (key == "KEEP_STATE") ok = as_int(&p->keep_state);
    else if (key == "AUTOTUNE") ok = as_int(&p->autotune);
    else if (key == "STAGING") ok = as_int(&p->staging);
    else {
        *why = "unrecognised option '" + key + "'";
        return FR_ERR_PARSE;
    }
    if (!ok) {
        *why = "bad value '" + val + "' for '" + key + "'";
        return FR_ERR_PARSE;
    }
    return FR_OK;
}

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

thread_local std::string g_parse_error;

}  // namespace

namespace frg {
void set_global_error(const char* msg) { g_parse_error = msg ? msg : ""; }
}  // namespace frg

extern "C" {

int fr_abi_version(void) { return FR_ABI_VERSION; }

const char* fr_status_string(int status) {
    switch (status) {
        case FR_OK: return "ok";
        case FR_ERR_INVALID_ARG: return "invalid argument";
        case FR_ERR_CUDA: return "CUDA error";
        case FR_ERR_ALLOC: return "allocation failed";
        case FR_ERR_IO: return "I/O error";
        case FR_ERR_PARSE: return "parse error";
        case FR_ERR_STATE: return "call out of order";
        case FR_ERR_NUMERIC: return "NaN/Inf in the solver";
        default: return "unknown status";
    }
}

const char* fr_last_error(const fr_handle* h) {
    if (!h) return g_parse_error.c_str();
    return h->err.c_str();
}

int fr_params_default(fr_params* p) {
    if (!p) return FR_ERR_INVALID_ARG;
    std::memset(p, 0, sizeof(*p));
    // values of the reference's params.ini (params.ini:1-25); Params defaults
    // reset_iter = -1, verbosity = 0 (params.hpp:11-12)
    p->volume_dims[0] = 193;
    p->volume_dims[1] = 229;
    p->volume_dims[2] = 193;
    p->volume_size[0] = p->volume_size[1] = p->volume_size[2] = 1.f;
    p->no_labels = 6;
    p->alpha = 0.004f;
    p->max_iter = 2048;
    p->max_update_norm = -1e-10f;
    p->rho_0 = 1.f;
    p->tau = 0.2f;
    p->w_reg = 0.2f;
    p->reset_iter = -1;
    p->p = 2.f;
    p->C = 0.25f;
    p->verbosity = 0;
    p->solver = FR_SOLVER_REFERENCE;
    p->smooth_sigma = 1.5f;
    p->smooth_width = 7;
    p->damping = 0.9f;
    p->step = 0.5f;
    p->keep_state = 0;
    p->autotune = 1;
    p->staging = 0;
    return FR_OK;
}

int fr_params_parse_ini(const char* text, fr_params* p) {
    g_parse_error.clear();
    if (!text || !p) {
        g_parse_error = "NULL argument";
        return FR_ERR_INVALID_ARG;
    }
    std::istringstream in(text);
    std::string line;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        line = trim(line);
        if (line.empty()) continue;
        if (line.front() == '[' && line.back() == ']') continue;  // section headers are ignored
        size_t eq = line.find('=');
        if (eq == std::string::npos) {
            g_parse_error = "line " + std::to_string(lineno) + ": expected KEY=VALUE";
            return FR_ERR_PARSE;
        }
        std::string why;
        int rc = set_key(p, trim(line.substr(0, eq)), trim(line.substr(eq + 1)), &why);
        if (rc != FR_OK) {
            g_parse_error = "line " + std::to_string(lineno) + ": " + why;
            return rc;
        }
    }
    return FR_OK;
}

int fr_params_load_ini(const char* path, fr_params* p) {
    g_parse_error.clear();
    if (!path || !p) {
        g_parse_error = "NULL argument";
        return FR_ERR_INVALID_ARG;
    }
    std::ifstream f(path);
    if (!f) {
        g_parse_error = std::string("cannot open ") + path;
        return FR_ERR_IO;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    return fr_params_parse_ini(ss.str().c_str(), p);
}

int fr_create(const fr_params* p, fr_handle** out) {
    if (!out) return FR_ERR_INVALID_ARG;
    *out = nullptr;
    fr_handle* h = new (std::nothrow) fr_handle();
    if (!h) return FR_ERR_ALLOC;
    int rc = check_params(h, p);
    if (rc != FR_OK) {
        g_parse_error = h->err;
        delete h;
        return rc;
    }
    h->P = *p;
    if (cudaGetDevice(&h->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess) {
        cudaGetLastError();
        g_parse_error = "no CUDA device available";
        delete h;
        return FR_ERR_CUDA;
    }
    *out = h;
    return FR_OK;
}

int fr_destroy(fr_handle* h) {
    if (!h) return FR_ERR_INVALID_ARG;
    cudaDeviceSynchronize();
    release(h);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    delete h;
    return FR_OK;
}

int fr_begin(fr_handle* h, const fr_pair* pairs, int n_pairs, void* stream) {
    if (!h) return FR_ERR_INVALID_ARG;
    return begin(h, pairs, n_pairs, (cudaStream_t)stream);
}

int fr_step(fr_handle* h, int iter, float t, void* stream) {
    if (!h) return FR_ERR_INVALID_ARG;
    if (!h->have_state) return fail(h, FR_ERR_STATE, "fr_step before fr_begin");
    if (iter < 1 || iter > h->trace_cap) return fail(h, FR_ERR_INVALID_ARG, "iter %d outside [1, %d]", iter, h->trace_cap);
    if (!(t > 0.f)) return fail(h, FR_ERR_INVALID_ARG, "t must be > 0");
    int rc = launch_iter(h, iter, t, (cudaStream_t)stream);
    if (rc == FR_OK) {
        h->last_iter = iter;
        h->stats_ready = false;
        h->last_stream = (cudaStream_t)stream;
    }
    return rc;
}

int fr_finish(fr_handle* h, void* stream) {
    if (!h) return FR_ERR_INVALID_ARG;
    if (!h->have_state) return fail(h, FR_ERR_STATE, "fr_finish before fr_begin");
    return finish(h, (cudaStream_t)stream);
}

int fr_register_batch(fr_handle* h, const fr_pair* pairs, int n_pairs, void* stream) {
    if (!h) return FR_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = begin(h, pairs, n_pairs, s);
    if (rc != FR_OK) return rc;
    rc = run_registration(h, s);
    if (rc != FR_OK && rc != FR_ERR_NUMERIC) return rc;
    int rc2 = finish(h, s);
    if (rc2 != FR_OK) return rc2;
    if (h->P.verbosity > 0) {
        int rc3 = host_stats(h);
        if (rc3 != FR_OK) return rc3;
        for (int p = 0; p < h->npairs; ++p) {
            const fr_stats& st = h->stats[p];
            printf("POST-REGISTRATION\nDICE COEFFICIENT\n");
            for (int l = 1; l < h->P.no_labels; ++l) printf("label %d: %g\n", l, st.dice[l]);
            printf("all labels: %g\n", st.dice_all);
        }
        fflush(stdout);
    }
    return rc;
}

int fr_register(fr_handle* h, float* img_T, int16_t* lab_T, float* img_S, int16_t* lab_S, void* stream) {
    if (!h) return FR_ERR_INVALID_ARG;
    fr_pair pr;
    pr.dims[0] = h->P.volume_dims[0];
    pr.dims[1] = h->P.volume_dims[1];
    pr.dims[2] = h->P.volume_dims[2];
    pr.img_T = img_T;
    pr.lab_T = lab_T;
    pr.img_S = img_S;
    pr.lab_S = lab_S;
    return fr_register_batch(h, &pr, 1, stream);
}

int fr_get_stats(fr_handle* h, int pair, fr_stats* out) {
    if (!h || !out) return FR_ERR_INVALID_ARG;
    if (!h->finished) return fail(h, FR_ERR_STATE, "no finished registration");
    if (pair < 0 || pair >= h->npairs) return fail(h, FR_ERR_INVALID_ARG, "pair %d outside [0, %d)", pair, h->npairs);
    int rc = host_stats(h);
    if (rc != FR_OK) return rc;
    *out = h->stats[pair];
    return FR_OK;
}

int fr_get_trace(fr_handle* h, int pair, float* norms, int64_t* voxels, int cap, int* n_out) {
    if (!h || cap < 0) return FR_ERR_INVALID_ARG;
    if (!h->have_state) return fail(h, FR_ERR_STATE, "no registration");
    if (pair < 0 || pair >= h->npairs) return fail(h, FR_ERR_INVALID_ARG, "pair %d outside [0, %d)", pair, h->npairs);
    FR_CUDA(h, cudaStreamSynchronize(h->last_stream));
    int stop = 0;
    FR_CUDA(h, cudaMemcpy(&stop, h->stop + pair, sizeof(int), cudaMemcpyDeviceToHost));
    const int n = stop ? stop : h->last_iter;
    std::vector<unsigned long long> tr((size_t)h->npairs * h->trace_cap);
    FR_CUDA(h, cudaMemcpy(tr.data(), h->trace, sizeof(unsigned long long) * tr.size(), cudaMemcpyDeviceToHost));
    const int m = std::min(n, cap);
    for (int i = 0; i < m; ++i) {
        float nrm;
        long long ip;
        decode_key(tr[(size_t)i * h->npairs + pair], &nrm, &ip);
        if (norms) norms[i] = nrm;
        if (voxels) voxels[i] = (int64_t)user_index(h->hpairs[pair], ip);
    }
    if (n_out) *n_out = n;
    return FR_OK;
}

static int field_ptrs(fr_handle* h, int pair, int which, float** bufs, int* ncomp, int* nbufs) {
    if (!h->have_state) return fail(h, FR_ERR_STATE, "no registration state");
    if (pair < 0 || pair >= h->npairs) return fail(h, FR_ERR_INVALID_ARG, "pair %d outside [0, %d)", pair, h->npairs);
    const bool ref = h->P.solver == FR_SOLVER_REFERENCE;
    switch (which) {
        case FR_FIELD_PSI:
            bufs[0] = h->psi;
            *ncomp = 3;
            *nbufs = 1;
            return FR_OK;
        case FR_FIELD_PSI_INV:
            if (!ref) return fail(h, FR_ERR_INVALID_ARG, "the sobolev solver keeps no psi_inv");
            bufs[0] = h->pinv[0];
            bufs[1] = h->pinv[1];
            *ncomp = 3;
            *nbufs = 2;
            return FR_OK;
        case FR_FIELD_V:
            bufs[0] = h->v[0];
            bufs[1] = h->v[1];
            *ncomp = 3;
            *nbufs = ref ? 2 : 1;
            return FR_OK;
        case FR_FIELD_RHO:
            if (!ref) return fail(h, FR_ERR_INVALID_ARG, "the sobolev solver keeps no density");
            bufs[0] = h->rho[0];
            bufs[1] = h->rho[1];
            *ncomp = 1;
            *nbufs = 2;
            return FR_OK;
        default:
            return fail(h, FR_ERR_INVALID_ARG, "unknown field %d", which);
    }
}

int fr_get_field(fr_handle* h, int pair, int which, float* d_buf, void* stream) {
    if (!h || !d_buf) return FR_ERR_INVALID_ARG;
    float* bufs[2] = {nullptr, nullptr};
    int ncomp = 0, nbufs = 0;
    int rc = field_ptrs(h, pair, which, bufs, &ncomp, &nbufs);
    if (rc != FR_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int sel = 0;
    if (nbufs == 2) {
        FR_CUDA(h, cudaStreamSynchronize(h->last_stream));
        int stop = 0;
        FR_CUDA(h, cudaMemcpy(&stop, h->stop + pair, sizeof(int), cudaMemcpyDeviceToHost));
        sel = (stop ? stop : h->last_iter) & 1;
    }
    const Pair& P = h->hpairs[pair];
    const size_t nu = (size_t)P.X * P.Y * P.Z;  // caller's (unpadded) plane
    for (int c = 0; c < ncomp; ++c)
        FR_CUDA(h, cudaMemcpy2DAsync(d_buf + c * nu, sizeof(float) * P.X, bufs[sel] + c * h->NT + P.off,
                                     sizeof(float) * P.Xp, sizeof(float) * P.X, (size_t)P.Y * P.Z,
                                     cudaMemcpyDeviceToDevice, s));
    return FR_OK;
}

int fr_set_field(fr_handle* h, int pair, int which, const float* d_buf, void* stream) {
    if (!h || !d_buf) return FR_ERR_INVALID_ARG;
    float* bufs[2] = {nullptr, nullptr};
    int ncomp = 0, nbufs = 0;
    int rc = field_ptrs(h, pair, which, bufs, &ncomp, &nbufs);
    if (rc != FR_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const Pair& P = h->hpairs[pair];
    const size_t nu = (size_t)P.X * P.Y * P.Z;  // caller's (unpadded) plane
    for (int b = 0; b < nbufs; ++b)
        for (int c = 0; c < ncomp; ++c)
            FR_CUDA(h, cudaMemcpy2DAsync(bufs[b] + c * h->NT + P.off, sizeof(float) * P.Xp, d_buf + c * nu,
                                         sizeof(float) * P.X, sizeof(float) * P.X, (size_t)P.Y * P.Z,
                                         cudaMemcpyDeviceToDevice, s));
    h->stats_ready = false;
    return FR_OK;
}

int fr_time_kernels(fr_handle* h, int iters, float* ms, int* n_kernels, void* stream) {
    if (!h || !ms || iters < 1) return FR_ERR_INVALID_ARG;
    if (!h->have_state) return fail(h, FR_ERR_STATE, "fr_time_kernels before fr_begin");
    cudaStream_t s = (cudaStream_t)stream;
    const int nk = kernels_per_iter(h);
    cudaEvent_t ev[6] = {};
    int rc = FR_OK;
    for (int k = 0; k <= nk && rc == FR_OK; ++k)
        if (cudaEventCreate(&ev[k]) != cudaSuccess) rc = fail(h, FR_ERR_CUDA, "fr_time_kernels: cudaEventCreate failed");
    std::vector<double> acc(nk, 0.0);
    std::vector<float> ts = t_schedule(h->P);
    for (int it = 1; it <= iters && rc == FR_OK; ++it) {
        // iterations cycle through the schedule; every kernel reads what it would read
        const int slot = 1 + (it - 1) % std::max(h->trace_cap, 1);
        const float t = ts.empty() ? h->P.alpha : ts[(slot - 1) % ts.size()];
        rc = launch_iter(h, slot, t, s, ev);
        if (rc != FR_OK) break;
        cudaError_t e = cudaEventSynchronize(ev[nk]);
        for (int k = 0; k < nk && e == cudaSuccess; ++k) {
            float m = 0.f;
            e = cudaEventElapsedTime(&m, ev[k], ev[k + 1]);
            acc[k] += m;
        }
        if (e != cudaSuccess) rc = fail(h, FR_ERR_CUDA, "fr_time_kernels: %s", cudaGetErrorString(e));
        h->last_iter = slot;
    }
    for (int k = 0; k <= nk; ++k)
        if (ev[k]) cudaEventDestroy(ev[k]);
    if (rc != FR_OK) return rc;
    rc = check_device_error(h);
    if (rc != FR_OK) return rc;
    for (int k = 0; k < nk; ++k) ms[k] = (float)(acc[k] / iters);
    if (n_kernels) *n_kernels = nk;
    h->stats_ready = false;
    return FR_OK;
}

int fr_warp(const float* d_pos, const float* d_img, const int16_t* d_lab, const int dims[3], float* d_out,
            int16_t* d_out_lab, void* stream) {
    g_parse_error.clear();
    if (!d_pos || !d_img || !d_out || !dims) {
        g_parse_error = "fr_warp: NULL argument";
        return FR_ERR_INVALID_ARG;
    }
    if (d_out_lab && !d_lab) {
        g_parse_error = "fr_warp: d_out_lab given without d_lab";
        return FR_ERR_INVALID_ARG;
    }
    if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) {
        g_parse_error = "fr_warp: dims must be >= 1";
        return FR_ERR_INVALID_ARG;
    }
    Pair P{};
    P.X = dims[0];
    P.Y = dims[1];
    P.Z = dims[2];
    P.Xp = P.X;  // the caller's unpadded layout
    P.N = (long long)P.X * P.Y * P.Z;
    P.off = 0;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto aligned = [](const void* p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) == 0; };
    const bool vec2 = P.N % 2 == 0 && frg::fits_index32(P.X, P.Y, P.Z) && aligned(d_pos, 8) && aligned(d_out, 8) &&
                      (!d_out_lab || aligned(d_out_lab, 4));
    const void* fn = vec2 ? (const void*)frg::warp2_kernel : (const void*)frg::warp_kernel;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0);
    const long long want = ((vec2 ? P.N / 2 : P.N) + 255) / 256;
    int grid = (int)std::max(1LL, std::min<long long>(want, (long long)std::max(per_sm, 1) * std::max(sms, 1)));
    if (vec2)
        frg::warp2_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_pos, d_img, d_lab, d_out, d_out_lab, P.X, P.Y, P.Z);
    else
        frg::warp_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_pos, d_img, d_lab, d_out, d_out_lab, P);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_parse_error = std::string("fr_warp: ") + cudaGetErrorString(e);
        return FR_ERR_CUDA;
    }
    return FR_OK;
}

static int field_op_check(const void* a, const void* b, const void* c, const int dims[3], const char* who) {
    g_parse_error.clear();
    if (!a || !b || !c || !dims) {
        g_parse_error = std::string(who) + ": NULL argument";
        return FR_ERR_INVALID_ARG;
    }
    if (!frg::fits_index32(dims[0], dims[1], dims[2])) {
        g_parse_error = std::string(who) + ": dims must be >= 1 with N + 2 X Y + 2 X + 2 <= 2^31-1";
        return FR_ERR_INVALID_ARG;
    }
    return FR_OK;
}

static int field_op_launch(const void* fn, long long work, const char* who, void (*launch)(int grid, void* ctx),
                           void* ctx) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0);
    const int grid =
        (int)std::max(1LL, std::min<long long>((work + 255) / 256, (long long)std::max(per_sm, 1) * std::max(sms, 1)));
    launch(grid, ctx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_parse_error = std::string(who) + ": " + cudaGetErrorString(e);
        return FR_ERR_CUDA;
    }
    return FR_OK;
}

int fr_set_pair_w_reg(fr_handle* h, const float* w_reg, int n) {
    if (!h) return FR_ERR_INVALID_ARG;
    h->err.clear();
    if (!w_reg || n <= 0) {
        h->pair_w_reg.clear();
        return FR_OK;
    }
    for (int p = 0; p < n; ++p)
        if (!std::isfinite(w_reg[p])) return fail(h, FR_ERR_INVALID_ARG, "w_reg[%d] is not finite", p);
    h->pair_w_reg.assign(w_reg, w_reg + n);
    return FR_OK;
}

int fr_tile_shape(const fr_handle* h, int k, int* depth, int* blocks_per_sm) {
    if (!h || !depth || !blocks_per_sm || k < 0 || k > 2) return FR_ERR_INVALID_ARG;
    if (!h->block) return FR_ERR_STATE;
    const TileSet& t = h->ts[active_roles(h)[k]];
    *depth = t.shape.depth;
    *blocks_per_sm = t.shape.bps;
    return FR_OK;
}

int fr_tile_staging(const fr_handle* h, int k, int* tma) {
    if (!h || !tma || k < 0 || k > 2) return FR_ERR_INVALID_ARG;
    if (!h->block) return FR_ERR_STATE;
    *tma = h->ts[active_roles(h)[k]].shape.variant;
    return FR_OK;
}

int fr_estimate_inverse(const float* d_psi, float* d_psi_inv, const int dims[3], int sweeps, void* stream) {
    int rc = field_op_check(d_psi, d_psi_inv, d_psi_inv, dims, "fr_estimate_inverse");
    if (rc != FR_OK) return rc;
    if (sweeps < 0) {
        g_parse_error = "fr_estimate_inverse: sweeps must be >= 0";
        return FR_ERR_INVALID_ARG;
    }
    struct Ctx {
        const float* psi;
        float* pinv;
        const int* d;
        int sweeps;
        cudaStream_t s;
    } c{d_psi, d_psi_inv, dims, sweeps, (cudaStream_t)stream};
    return field_op_launch(
        (const void*)frg::estimate_inverse_kernel, (long long)dims[0] * dims[1] * dims[2], "fr_estimate_inverse",
        [](int grid, void* p) {
            Ctx* c = (Ctx*)p;
            frg::estimate_inverse_kernel<<<grid, 256, 0, c->s>>>(c->psi, c->pinv, c->d[0], c->d[1], c->d[2], c->sweeps);
        },
        &c);
}

int fr_interpolate_field(const float* d_field, const float* d_pos, const int dims[3], float* d_out, void* stream) {
    int rc = field_op_check(d_field, d_pos, d_out, dims, "fr_interpolate_field");
    if (rc != FR_OK) return rc;
    struct Ctx {
        const float* f;
        const float* pos;
        float* out;
        const int* d;
        cudaStream_t s;
    } c{d_field, d_pos, d_out, dims, (cudaStream_t)stream};
    return field_op_launch(
        (const void*)frg::interpolate_field_kernel, (long long)dims[0] * dims[1] * dims[2], "fr_interpolate_field",
        [](int grid, void* p) {
            Ctx* c = (Ctx*)p;
            frg::interpolate_field_kernel<<<grid, 256, 0, c->s>>>(c->f, c->pos, c->out, c->d[0], c->d[1], c->d[2]);
        },
        &c);
}

}  // extern "C"
