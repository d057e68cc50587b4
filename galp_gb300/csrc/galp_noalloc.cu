// galp_noalloc.cu -- label propagation for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code that runs under an external allocator
// that owns all device memory, plugins loaded into a host framework that forbids
// allocation outside its pool, and latency-critical paths where an allocation (and
// its implicit synchronisation) is not acceptable.  galp_run_noalloc serves them.  It
// runs a different kernel from galp_run -- the single-pass tile kernel (lp_tile_kernel:
// counting, run bases by decoupled look-back and resolution in one launch per
// iteration) instead of the degree-bucketed count/scan/resolve pipeline -- with the
// same labels, iteration counts and change counts.  Every device buffer it needs --
// the copy of the graph, both label buffers, the tile schedule, the look-back status
// words and the control block -- lives in one file-scope static device array of
// kScratchBytes (12.5 MiB), which every GPU that loads the library holds until the
// process exits.  It calls no cudaMalloc, cudaFree or other allocating routine, on
// the device or the host.
//
// Limits: n <= GALP_NOALLOC_MAX_VERTICES, m <= GALP_NOALLOC_MAX_ENTRIES, and no vertex
// above 2048 neighbours (those need the global-table path, whose tables are sized per
// graph).  Larger graphs are rejected with GALP_EUNSUPPORTED.
//
// Set-up: every call looks up the device address of the static array with
// cudaGetSymbolAddress (the array's name is a host-side stand-in in host code); the
// first call on a device, or the first after the device's context was reset, also
// clears the status words.  A call
// must never be made on a stream that is being captured: it copies from pageable host
// memory and synchronises the stream, so it checks and returns GALP_EUNSUPPORTED.
// All calls on a device share the one array and the array keeps the last call's
// contents; each call clears or overwrites what it reads.  Calls that overlap on the
// GPU race on it; calls from one process are serialised per device, and every call
// (on success and on error) waits for the work it queued before it returns.
//
// Failure detection: every look-back wait is bounded (kSpinLimit polls by default);
// a wait that runs out sets an error bit and the kernel returns, and the call reports
// GALP_ETIMEOUT.  galp_debug_noalloc_lookback (tests only) lowers the bound and makes
// the waits expect a status epoch that no tile publishes, so that they run out.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/galp.h"

// The kernels are compiled into this translation unit with internal linkage.
namespace {
#include "lp_kernels.cuh"
}  // namespace

namespace {

using galp::Ctl;
using galp::IterArgs;
using galp::TileSmem;

constexpr int64_t kMaxV = GALP_NOALLOC_MAX_VERTICES;
constexpr int64_t kMaxE = GALP_NOALLOC_MAX_ENTRIES;

// Layout of the scratch array (byte offsets, each 256-aligned).
constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffNbr = 0;
constexpr size_t kOffOff = al(kOffNbr + sizeof(int32_t) * kMaxE);
constexpr size_t kOffLab0 = al(kOffOff + sizeof(int64_t) * (kMaxV + 1));
constexpr size_t kOffLab1 = al(kOffLab0 + sizeof(int32_t) * kMaxV);
constexpr size_t kOffVpos = al(kOffLab1 + sizeof(int32_t) * kMaxV);
constexpr size_t kOffTileV0 = al(kOffVpos + sizeof(uint16_t) * kMaxV);
constexpr size_t kOffTileBig = al(kOffTileV0 + sizeof(int32_t) * (kMaxV + 1));
constexpr size_t kOffTileUsed = al(kOffTileBig + sizeof(int32_t) * kMaxV);
constexpr size_t kOffStatus = al(kOffTileUsed + sizeof(uint16_t) * kMaxV);
constexpr size_t kOffCtl = al(kOffStatus + sizeof(unsigned long long) * kMaxV);
constexpr size_t kOffBad = al(kOffCtl + sizeof(Ctl));
constexpr size_t kScratchBytes = al(kOffBad + sizeof(int));

}  // namespace

// The scratch.  Device code could name it directly; host code only uses the address
// returned by cudaGetSymbolAddress (the name is a host-side stand-in there).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

constexpr int kMaxDevices = 64;

// failure-detection test hook (galp_debug_noalloc_lookback)
std::mutex g_debug_mu;
long long g_spin_limit = galp::kSpinLimit;
bool g_wait_unset = false;

struct DeviceState {
    std::mutex mu;
    unsigned char *base = nullptr;  // device address of g_noalloc_scratch on this device
    unsigned epoch = 0;             // last look-back epoch used on this device
    int grid = 0;                   // persistent grid of the tile kernel
};
DeviceState g_dev[kMaxDevices];

// Every call, with the device current: the array's device address and the tile
// kernel's shared-memory opt-in.  When the address differs from the one recorded (first
// call on the device, or a new context after a device reset reloaded the module), also
// the tile kernel's grid and a cleared status area.
int setup_device(int dev, DeviceState &D, cudaStream_t st)
{
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return GALP_ECUDA;
    // a context-level attribute: set on every call, so a reset context gets it again
    if (cudaFuncSetAttribute(galp::lp_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(TileSmem)) != cudaSuccess)
        return GALP_ECUDA;
    if (D.base == (unsigned char *)ptr) return GALP_OK;
    D.base = nullptr;
    D.epoch = 0;
    int sms = 0, occ = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GALP_ECUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, galp::lp_tile_kernel, galp::kTB, sizeof(TileSmem)) !=
        cudaSuccess)
        return GALP_ECUDA;
    unsigned char *b = (unsigned char *)ptr;
    if (cudaMemsetAsync(b + kOffStatus, 0, sizeof(unsigned long long) * kMaxV, st) != cudaSuccess) return GALP_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return GALP_ECUDA;
    D.grid = (occ > 0 ? occ : 1) * sms;
    D.base = b;
    return GALP_OK;
}

// Streams a host-generated array to the device through a fixed stack buffer.
template <class T, int CAP = 2048>
struct Stager {
    T buf[CAP];
    int cnt = 0;
    int64_t at = 0;  // element index of buf[0] in the destination
    T *dst;
    cudaStream_t st;
    cudaError_t err = cudaSuccess;
    Stager(T *d, cudaStream_t s) : dst(d), st(s) {}
    void push(T x)
    {
        buf[cnt++] = x;
        if (cnt == CAP) flush();
    }
    void flush()
    {
        // pageable source: the call returns once the buffer has been staged
        if (cnt && err == cudaSuccess) err = cudaMemcpyAsync(dst + at, buf, sizeof(T) * cnt, cudaMemcpyHostToDevice, st);
        at += cnt;
        cnt = 0;
    }
};

}  // namespace

extern "C" int galp_debug_noalloc_lookback(int64_t spin_limit, int32_t wait_unset)
{
    std::lock_guard<std::mutex> lock(g_debug_mu);
    g_spin_limit = spin_limit > 0 ? (long long)spin_limit : galp::kSpinLimit;
    g_wait_unset = wait_unset != 0;
    return GALP_OK;
}

extern "C" int galp_run_noalloc(const galp_csr *g, int32_t niter, int32_t early_exit, int32_t *labels_out,
                                galp_stats *stats, void *stream)
{
    if (!g || niter < 0 || niter > GALP_MAX_ITERS || !g->offsets || g->n < 0 || g->m < 0) return GALP_EINVAL;
    if (g->n > 0 && !labels_out) return GALP_EINVAL;
    if (g->m > 0 && !g->neighbors) return GALP_EINVAL;
    if (g->n > kMaxV || g->m > kMaxE) return GALP_EUNSUPPORTED;
    if (g->offsets[0] != 0 || g->offsets[g->n] != g->m) return GALP_EFORMAT;
    for (int64_t v = 0; v < g->n; ++v) {
        const int64_t deg = g->offsets[v + 1] - g->offsets[v];
        if (deg < 0) return GALP_EFORMAT;
        if (deg > galp::kTileSlots) return GALP_EUNSUPPORTED;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GALP_ENODEV;
    if (dev < 0 || dev >= kMaxDevices) return GALP_EUNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    // never on a capturing stream (pageable copies and stream synchronisation)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        (void)cudaGetLastError();
        return GALP_EUNSUPPORTED;
    }
    long long spin_limit;
    bool wait_unset;
    {
        std::lock_guard<std::mutex> lock(g_debug_mu);
        spin_limit = g_spin_limit;
        wait_unset = g_wait_unset;
    }
    DeviceState &D = g_dev[dev];
    std::lock_guard<std::mutex> lock(D.mu);
    (void)cudaGetLastError();  // an earlier, unrelated runtime error must not be reported as ours
    // after work has been queued, every error return first waits for it (best effort), so
    // that no kernel of this call still uses the shared array when the next call starts
    auto fail = [&](int code) {
        (void)cudaStreamSynchronize(st);
        (void)cudaGetLastError();
        return code;
    };
    int rc = setup_device(dev, D, st);
    if (rc) return fail(rc);

    const int64_t n = g->n, m = g->m;
    unsigned char *B = D.base;
    int32_t *d_nbr = (int32_t *)(B + kOffNbr);
    int64_t *d_off = (int64_t *)(B + kOffOff);
    int32_t *lab[2] = {(int32_t *)(B + kOffLab0), (int32_t *)(B + kOffLab1)};
    uint16_t *d_vpos = (uint16_t *)(B + kOffVpos);
    int32_t *d_tile_v0 = (int32_t *)(B + kOffTileV0);
    int32_t *d_tile_big = (int32_t *)(B + kOffTileBig);
    uint16_t *d_tile_used = (uint16_t *)(B + kOffTileUsed);
    unsigned long long *d_status = (unsigned long long *)(B + kOffStatus);
    Ctl *d_ctl = (Ctl *)(B + kOffCtl);
    int *d_bad = (int *)(B + kOffBad);

    // graph
    if (m && cudaMemcpyAsync(d_nbr, g->neighbors, sizeof(int32_t) * m, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return fail(GALP_ECUDA);
    if (cudaMemcpyAsync(d_off, g->offsets, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return fail(GALP_ECUDA);

    // tile schedule (same packing rule as the allocating path), streamed to the device
    int64_t ntiles = 0;
    int32_t last_v = -1;
    {
        Stager<uint16_t> vpos(d_vpos, st);
        Stager<int32_t> tv0(d_tile_v0, st), tbig(d_tile_big, st);
        Stager<uint16_t> tused(d_tile_used, st);
        int cur = 0, nvt = 0;
        int64_t tstart = 0;
        auto close = [&](int64_t vend) {
            if (vend > tstart) {
                tv0.push((int32_t)tstart);
                tbig.push(-1);
                tused.push((uint16_t)cur);
                ++ntiles;
            }
            tstart = vend;
            cur = 0;
            nvt = 0;
        };
        for (int64_t v = 0; v < n; ++v) {
            const int deg = (int)(g->offsets[v + 1] - g->offsets[v]);
            if (deg > 0) last_v = (int32_t)v;
            auto place = [&](int c, int &pos, int &end) {
                if (deg == 0) {
                    pos = c;
                    end = c;
                } else if (deg <= galp::kSmallMax) {
                    pos = ((c & 31) + deg > 32) ? ((c + 31) & ~31) : c;
                    end = pos + deg;
                } else {
                    pos = (c + 31) & ~31;
                    end = pos + ((deg + 31) & ~31);
                }
            };
            int pos, end;
            place(cur, pos, end);
            if (nvt == galp::kTileV || end > galp::kTileSlots) {
                close(v);
                place(0, pos, end);
            }
            vpos.push((uint16_t)pos);
            cur = end;
            nvt++;
        }
        close(n);
        tv0.push((int32_t)n);
        vpos.flush();
        tv0.flush();
        tbig.flush();
        tused.flush();
        if (vpos.err || tv0.err || tbig.err || tused.err) return fail(GALP_ECUDA);
    }

    // neighbours in range before any iteration reads labels through them
    if (cudaMemsetAsync(d_bad, 0, sizeof(int), st) != cudaSuccess) return fail(GALP_ECUDA);
    if (m) galp::validate_kernel<<<256, 256, 0, st>>>(d_nbr, m, n, d_bad);
    if (cudaGetLastError() != cudaSuccess) return fail(GALP_ECUDA);
    int bad = 0;
    if (cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return fail(GALP_ECUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(GALP_ECUDA);
    if (bad) return fail(GALP_EFORMAT);

    const long long thr = early_exit ? (long long)std::floor((double)n * 1e-5) : -1;
    if (n) galp::init_labels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(lab[0], n);
    galp::init_ctl_kernel<<<1, 1, 0, st>>>(d_ctl, thr, niter);
    if (cudaGetLastError() != cudaSuccess) return fail(GALP_ECUDA);
    IterArgs a{};
    a.nbr = d_nbr;
    a.off = d_off;
    a.vpos = d_vpos;
    a.tile_v0 = d_tile_v0;
    a.tile_big = d_tile_big;
    a.tile_used = d_tile_used;
    a.ntiles = (int32_t)ntiles;
    a.last_v = last_v;
    a.status = d_status;
    a.ctl = d_ctl;
    a.spin_limit = spin_limit;
    a.wait_xor = wait_unset ? 1u : 0u;
    const int grid = (int)(ntiles < D.grid ? ntiles : D.grid);
    for (int it = 0; it < niter; ++it) {
        a.lab_in = lab[it & 1];
        a.lab_out = lab[(it + 1) & 1];
        // the test hook clears the status words every iteration, so that only this
        // iteration's epoch is present and epoch ^ 1 is published by no tile
        if (++D.epoch > (unsigned)galp::kEpochMask || wait_unset) {
            if (D.epoch > (unsigned)galp::kEpochMask) D.epoch = 1;
            if (cudaMemsetAsync(d_status, 0, sizeof(unsigned long long) * kMaxV, st) != cudaSuccess)
                return fail(GALP_ECUDA);
        }
        a.epoch = D.epoch;
        if (cudaMemsetAsync(&d_ctl->ticket, 0, sizeof(unsigned long long), st) != cudaSuccess) return fail(GALP_ECUDA);
        if (grid > 0) galp::lp_tile_kernel<<<grid, galp::kTB, sizeof(TileSmem), st>>>(a);
        galp::finalize_kernel<<<1, 1, 0, st>>>(d_ctl);
        if (cudaGetLastError() != cudaSuccess) return fail(GALP_ECUDA);
    }
    Ctl c;
    if (cudaMemcpyAsync(&c, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st) != cudaSuccess) return fail(GALP_ECUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(GALP_ECUDA);
    if (n && cudaMemcpyAsync(labels_out, lab[c.iter & 1], sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return fail(GALP_ECUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(GALP_ECUDA);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->iters_run = c.iter;
        stats->err = c.err;
        stats->runs_last = c.N;
        for (int i = 0; i < GALP_MAX_ITERS; ++i) stats->updates[i] = (int64_t)c.counts[i];
        stats->h2d_bytes = (int64_t)(sizeof(int32_t) * m + sizeof(int64_t) * (n + 1));
        stats->d2h_bytes = (int64_t)sizeof(int32_t) * n;
    }
    return (c.err & galp::kErrLookback) ? GALP_ETIMEOUT : GALP_OK;
}
