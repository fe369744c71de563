// i2_noalloc.cu -- the disjoint ("not neighbours") pair class with relative error control, run
// without allocating anything: every scratch buffer lives in one file-scope device array.
//
// Who needs this: callers that cannot call cudaMalloc / cudaFree.  Examples are plugins
// running inside a host application that reserves the GPU's memory up front for its own pool
// (an allocation there fails or takes memory the host has already promised elsewhere), and
// time-critical loops where an allocation is not allowed because cudaMalloc / cudaFree can
// synchronise the device and take unbounded time.  Such a caller passes its own device
// buffers for the inputs and outputs; the per-cell panel records, per-pair sums, active lists
// and counters go into the static array below.
//
// The array's size is fixed at build time (limits below) and every GPU that loads this
// library holds it until the process exits.  All calls share it and it keeps the last call's
// contents: each call clears the counters that must start at zero and overwrites the rest
// before reading it.  Calls that overlap on the GPU (two streams, or two host threads whose
// calls run at the same time) race on the array and corrupt each other's results.
#include "integrator2_gb300.h"
#include "i2_engine.h"

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

namespace {

constexpr int kMaxCells = I2_NOALLOC_MAX_CELLS;
constexpr int kMaxPairs = I2_NOALLOC_MAX_PAIRS;
constexpr int kMaxDevices = 64;

// layout of the scratch array (every region starts on a 256-byte boundary)
constexpr size_t kPanelsOff = 0;
constexpr size_t kCurOff = kPanelsOff + sizeof(i2::Panel) * (size_t)kMaxCells;
constexpr size_t kFinAOff = kCurOff + 5 * sizeof(double) * (size_t)kMaxPairs;
constexpr size_t kFinBOff = kFinAOff + 5 * sizeof(double) * (size_t)kMaxPairs;
constexpr size_t kRawOff = kFinBOff + 5 * sizeof(double) * (size_t)kMaxPairs;
constexpr size_t kStopOff = kRawOff + 4 * sizeof(double) * (size_t)kMaxPairs;
constexpr size_t kActAOff = kStopOff + sizeof(int) * (size_t)kMaxPairs;
constexpr size_t kActBOff = kActAOff + sizeof(int) * (size_t)kMaxPairs;
constexpr size_t kCntOff = kActBOff + sizeof(int) * (size_t)kMaxPairs;
constexpr size_t kCntInts = 64;  // cnt[0..15] active counts per level, cnt[16] deepest level
constexpr size_t kScratchBytes = kCntOff + sizeof(int) * kCntInts;
static_assert(kCurOff % 256 == 0 && kFinAOff % 256 == 0 && kFinBOff % 256 == 0 && kRawOff % 256 == 0 && kStopOff % 256 == 0 &&
                  kActAOff % 256 == 0 && kActBOff % 256 == 0 && kCntOff % 256 == 0,
              "scratch regions are 256-byte aligned");

// the scratch array; in host code this name is only a handle for cudaGetSymbolAddress
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// The array's device address belongs to a CUDA context, not to a device ordinal: a host
// application may run its own driver-API context on a device, and a cudaDeviceReset makes a new
// primary context.  The set-up below therefore runs once per context (normally once per device,
// for its primary context), with that context current, and is cached under the context's ID
// (cuCtxGetId: unique for the life of the process, unlike a handle, which can be reused after
// its context is destroyed).
struct Setup {
    unsigned long long id;
    void *ptr;
    int sms;
};
constexpr int kMaxSetups = 4 * kMaxDevices;
std::mutex g_setup_mutex;
Setup g_setup[kMaxSetups] = {};
int g_nsetup = 0, g_next = 0;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (no libcuda link)
using CtxGetCurrentFn = int (*)(void **);
using CtxGetIdFn = int (*)(void *, unsigned long long *);
void *driver_fn(const char *name)
{
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess || q != cudaDriverEntryPointSuccess)
        return nullptr;
    return f;
}

// the ID of the context current on this thread; false when there is none (or no driver support)
bool current_context_id(unsigned long long &id)
{
    static const CtxGetCurrentFn get = reinterpret_cast<CtxGetCurrentFn>(driver_fn("cuCtxGetCurrent"));
    static const CtxGetIdFn get_id = reinterpret_cast<CtxGetIdFn>(driver_fn("cuCtxGetId"));
    void *ctx = nullptr;
    if (!get || !get_id || get(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, &id) == 0;
}

// with device dev current: the device address of the array in the current context and the SM count
i2_status device_setup(int dev, void **ptr, int *sms, std::string &err)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = 0;
    bool have_id = current_context_id(id);
    if (have_id)
        for (int k = 0; k < g_nsetup; ++k)
            if (g_setup[k].id == id) {
                *ptr = g_setup[k].ptr;
                *sms = g_setup[k].sms;
                return I2_OK;
            }
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);  // makes the device's primary context current if none was
    if (e != cudaSuccess || !p) {
        err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
        return I2_ERR_CUDA;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        err = "cannot read the SM count";
        return I2_ERR_CUDA;
    }
    if (!have_id) have_id = current_context_id(id);
    if (have_id) {  // without an ID (no driver entry point) the lookup simply repeats on every call
        const int k = g_nsetup < kMaxSetups ? g_nsetup++ : (g_next++ % kMaxSetups);
        g_setup[k] = Setup{id, p, n};
    }
    *ptr = p;
    *sms = n;
    return I2_OK;
}

bool aligned(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

i2_status fail(i2_status s, const std::string &msg)
{
    i2::set_last_error(msg);
    return s;
}

} // namespace

extern "C" i2_status i2_not_neighbors_noalloc(const double *d_vertices, int32_t nv, const int32_t *d_cells, int32_t nc,
                                              const int32_t *d_pairs, int64_t n, double rel_tol, int32_t max_level,
                                              double *d_J, double *d_P, void *stream)
{
    if (nc < 1 || nc > kMaxCells)
        return fail(I2_ERR_INVALID_ARGUMENT, "cell count must be 1.." + std::to_string(kMaxCells) + " (static scratch limit)");
    if (n < 0 || n > kMaxPairs)
        return fail(I2_ERR_INVALID_ARGUMENT, "pair count must be 0.." + std::to_string(kMaxPairs) + " (static scratch limit)");
    if (nv < 3) return fail(I2_ERR_INVALID_ARGUMENT, "at least 3 vertices");
    if (!(rel_tol > 0.0 && rel_tol < 1.0)) return fail(I2_ERR_INVALID_ARGUMENT, "relative tolerance must be in (0, 1)");
    if (max_level < 1 || max_level > i2::kMaxLevel) return fail(I2_ERR_INVALID_ARGUMENT, "max level must be 1..5");
    if (!d_vertices || !d_cells || (n > 0 && (!d_pairs || !d_J || !d_P)))
        return fail(I2_ERR_INVALID_ARGUMENT, "null device pointer");
    if (!aligned(d_vertices, 8) || !aligned(d_cells, 4) || !aligned(d_pairs, 8) || !aligned(d_J, 8) || !aligned(d_P, 8))
        return fail(I2_ERR_INVALID_ARGUMENT, "misaligned device pointer (pairs need 8 bytes, cells 4, doubles 8)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(I2_ERR_CUDA, "no current CUDA device");
    if (dev < 0 || dev >= kMaxDevices) return fail(I2_ERR_UNSUPPORTED, "device ordinal above 63");
    void *base = nullptr;
    int sms = 0;
    std::string err;
    const i2_status st = device_setup(dev, &base, &sms, err);
    if (st != I2_OK) return fail(st, err);
    if (n == 0) {
        i2::set_last_error("");
        return I2_OK;
    }
    const cudaStream_t s = (cudaStream_t)stream;
    unsigned char *b = static_cast<unsigned char *>(base);

    // the library's 13-point rule (the reference's qf3D13)
    double coords[26], weights[13];
    int32_t order = 0;
    if (i2_quadrature_builtin(13, coords, weights, &order) != I2_OK) return fail(I2_ERR_CUDA, "built-in rule missing");
    i2::QuadTables Q;
    std::memset(&Q, 0, sizeof Q);
    Q.npts = 13;
    for (int g = 0; g < 13; ++g) {
        Q.L1[g] = coords[2 * g];
        Q.L2[g] = coords[2 * g + 1];
        Q.L3[g] = 1.0 - coords[2 * g] - coords[2 * g + 1];
        Q.w[g] = weights[g];
    }
    Q.order = order;
    Q.pow2p = (double)(1 << order);

    i2::RunConfig cfg;
    cfg.mode = i2::kAdaptiveRelative;
    cfg.tol = rel_tol;
    cfg.max_level = max_level;
    cfg.hard_tol = 0.0;

    i2::ClassArgs A;
    A.n = (int)n;
    A.pairs = reinterpret_cast<const int2 *>(d_pairs);
    A.cells = reinterpret_cast<const int3 *>(d_cells);
    A.panels = reinterpret_cast<const i2::Panel *>(b + kPanelsOff);
    A.cur = reinterpret_cast<double *>(b + kCurOff);
    A.fin_a = reinterpret_cast<double *>(b + kFinAOff);
    A.fin_b = reinterpret_cast<double *>(b + kFinBOff);
    A.raw4 = reinterpret_cast<double *>(b + kRawOff);
    A.stop = reinterpret_cast<int *>(b + kStopOff);
    A.act_a = reinterpret_cast<int *>(b + kActAOff);
    A.act_b = reinterpret_cast<int *>(b + kActBOff);
    A.cnt = reinterpret_cast<int *>(b + kCntOff);
    A.maxlev = A.cnt + 16;
    A.J3 = d_J;
    A.P = d_P;

    // counters start at zero; everything else is written before it is read
    if (cudaMemsetAsync(A.cnt, 0, sizeof(int) * kCntInts, s) != cudaSuccess) return fail(I2_ERR_CUDA, "counter reset failed");
    i2::launch_prepare_panels(nc, d_vertices, d_cells, const_cast<i2::Panel *>(A.panels), s);
    i2::launch_class_fp64(i2::kFar, A, Q, cfg, std::max(1, sms) * 8, s);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(I2_ERR_CUDA, std::string("launch failed: ") + cudaGetErrorString(e));
    i2::set_last_error("");
    return I2_OK;
}
