// pcsf_lpr_noalloc: a likelihood evaluation that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a
// likelihood: code running inside a host framework that owns every device
// allocation through its own pool (and forbids the CUDA allocator), callers on
// a latency-critical thread where cudaMalloc's implicit synchronisation is not
// acceptable, or processes running under a hard device-memory cap that is
// already committed.  For them this entry point evaluates lpr_leaves for a
// batch of regions at one tree scale using only (a) device state the engine
// created when it was made, (b) the caller's input and output buffers, and
// (c) one fixed scratch area compiled into this library.
//
// The scratch area is a file-scope __device__ array of PCSF_NOALLOC_SCRATCH_BYTES
// (24 MiB): every GPU that loads the library holds it until the process exits.
// In host code its name is only a host-side stand-in, so its device address
// is looked up with cudaGetSymbolAddress on the first call on each device, with
// that device current (a failed lookup is retried by the next call).  That first
// call should therefore come before any stream capture.  All calls share the one
// area and it keeps the previous call's contents: the parts that must start at
// a known value (the status key, the invalid-code slot, the engine's error flag)
// are set on every call, and calls whose work overlaps on the GPU (from several
// host threads or engines on one device) race on it -- serialise them.  The host
// side uses fixed static arrays for the work list, so concurrent calls from
// several host threads race there too.
#include <cmath>
#include <cstring>
#include <mutex>

#include "pcsf_internal.h"

namespace pcsf {

constexpr size_t NOALLOC_BYTES = size_t(24) << 20;
constexpr int NOALLOC_MAX_REGIONS = 32768;
constexpr int NOALLOC_MAX_WORK = 131072;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// host-side staging of the work list (fixed size, no allocation at call time)
static PSet h_ps[1];
static Request h_req[NOALLOC_MAX_REGIONS];
static WorkItem h_wi[NOALLOC_MAX_WORK];
static int32_t h_wib[NOALLOC_MAX_REGIONS + 1];
static int32_t h_out[NOALLOC_MAX_REGIONS];   // request -> region (short regions first, then long ones)

static std::mutex g_scratch_mu;
static void *g_scratch_ptr[NOALLOC_MAX_DEVICES];

// Device address of the scratch array on `device` (which must be current).  Only a
// successful lookup is kept, so a lookup that failed for a passing reason (a sticky
// error of earlier work, a call made during stream capture) is tried again next time.
static cudaError_t scratch_on(int device, unsigned char **out)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        cudaError_t ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (ce != cudaSuccess) {
            cudaGetLastError();   // do not leave the failed lookup as the thread's last error
            return ce;
        }
        g_scratch_ptr[device] = p;
    }
    *out = reinterpret_cast<unsigned char *>(g_scratch_ptr[device]);
    return cudaSuccess;
}

static size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace pcsf

using namespace pcsf;

// Engine internals needed here (defined in engine.cpp).
int pcsf_internal_noalloc_ctx(pcsf_engine *e, NoallocCtx *c);
int pcsf_internal_fail(pcsf_engine *e, int code, const char *msg);

extern "C" int pcsf_lpr_noalloc(pcsf_engine *e, int32_t model, double rho, int32_t n_regions,
                                const int64_t *col_offsets, const uint8_t *d_leaves, double *d_lpr, double *d_elpr)
{
    if (!e) return PCSF_EINVAL;
    NoallocCtx cx;
    int rc = pcsf_internal_noalloc_ctx(e, &cx);
    if (rc != PCSF_OK) return rc;
    if (!cx.has_models) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: this engine has no coding / noncoding models");
    if (cx.tc_direct)
        return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: engines made with PCSF_TC_DIRECT are not supported "
                                                  "(their pcsf_lpr returns tensor-core values)");
    if (cudaSetDevice(cx.device) != cudaSuccess) return pcsf_internal_fail(e, PCSF_ECUDA, "pcsf_lpr_noalloc: cudaSetDevice");
    if (model < 0 || model > 1) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: model must be 0 or 1");
    if (!(rho > 0.0) || !std::isfinite(rho)) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: rho must be > 0");
    if (n_regions < 0 || (n_regions > 0 && (!col_offsets || !d_lpr)))
        return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: null argument");
    if (n_regions > NOALLOC_MAX_REGIONS)
        return pcsf_internal_fail(e, PCSF_ERANGE, "pcsf_lpr_noalloc: more than 32768 regions in one call");
    if (n_regions == 0) return PCSF_OK;
    if (col_offsets[0] != 0) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: col_offsets[0] must be 0");
    const int64_t total_cols = col_offsets[n_regions];
    if (total_cols > 0 && !d_leaves) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: d_leaves is NULL");
    // every returned likelihood comes from the kernels pcsf_lpr uses for it: the SIMT
    // kernel with pcsf_lpr's summation and P(t) formation, or -- for a region whose
    // columns x (n_leaves - 2) reach the engine's threshold -- the float-float kernel on
    // the FP64 P(t)
    const int prec = cx.prec;
    const int TC = simt_tile_cols(prec, cx.nslots, cx.simt_tile);
    const int TCX = ff_tile_cols();
    const bool fp32 = prec != PCSF_PREC_FP64;
    const size_t es = fp32 ? 4 : 8;
    const size_t nbr = (size_t)cx.nbr;
    auto is_long = [&](int64_t nc) {
        return cx.ff_grid > 0 && nc > 0 && nc * (int64_t)std::max(cx.nl - 2, 1) >= cx.exact_min_units;
    };
    // requests: the short regions first, then the long ones; work items contiguous per request
    int nreq = 0, nwi = 0, nws = 0;
    bool any_short = false, any_long = false;
    for (int pass = 0; pass < 2; pass++) {
        for (int r = 0; r < n_regions; r++) {
            const int64_t c0 = col_offsets[r], c1 = col_offsets[r + 1];
            if (c1 < c0) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: col_offsets not non-decreasing");
            if (is_long(c1 - c0) != (pass == 1)) continue;
            (pass ? any_long : any_short) = true;
            const int tc = pass ? TCX : TC;
            h_req[nreq] = Request{r, model, 0, (uint32_t)c0, rho};
            h_out[nreq] = r;
            h_wib[nreq] = nwi;
            for (int64_t c = c0; c < c1; c += tc) {
                if (nwi >= NOALLOC_MAX_WORK)
                    return pcsf_internal_fail(e, PCSF_ERANGE, "pcsf_lpr_noalloc: more than 131072 column tiles in one call");
                h_wi[nwi++] = WorkItem{nreq, (int32_t)std::min<int64_t>(tc, c1 - c), c};
            }
            nreq++;
        }
        if (pass == 0) nws = nwi;
    }
    h_wib[nreq] = nwi;
    // scratch map: [status key, invalid-code slot][requests][request -> region][P set][P(t) in the
    // arithmetic type][diag(E) low parts][FP64 P(t)][float-float P(t)][work items][wi_begin][partials][elpr]
    const bool stage64 = fp32 && ((cx.pt64 && any_short) || any_long);   // FP64 formation needed
    const size_t split_bytes = any_long ? up256(nbr * 2 * K2 * sizeof(float)) : 0;   // float-float P set
    const size_t off_req = 256;
    const size_t off_out = off_req + up256(sizeof(Request) * (size_t)n_regions);
    const size_t off_ps = off_out + up256(sizeof(int32_t) * (size_t)n_regions);
    const size_t off_P = off_ps + 256;
    const size_t off_dlo = off_P + up256(nbr * K2 * es);
    const size_t off_stage = off_dlo + (fp32 ? up256(nbr * K * sizeof(float)) : 0);
    const size_t off_split = off_stage + (stage64 ? up256(nbr * K2 * sizeof(double)) : 0);
    const size_t off_wi = off_split + split_bytes;
    const size_t off_wib = off_wi + up256(sizeof(WorkItem) * (size_t)nwi);
    const size_t off_part = off_wib + up256(sizeof(int32_t) * (size_t)(n_regions + 1));
    const size_t off_elpr = off_part + up256(sizeof(double) * 2 * (size_t)std::max(nwi, 1));
    const size_t need = off_elpr + (d_elpr ? 0 : sizeof(double) * (size_t)n_regions);
    if (need > NOALLOC_BYTES)
        return pcsf_internal_fail(e, PCSF_ERANGE, "pcsf_lpr_noalloc: batch needs more than the 24 MiB static scratch area");
    unsigned char *sc = nullptr;
    cudaError_t ce = scratch_on(cx.device, &sc);
    if (ce != cudaSuccess) return pcsf_internal_fail(e, PCSF_ECUDA, "pcsf_lpr_noalloc: cudaGetSymbolAddress failed");
    h_ps[0] = PSet{model, 0, rho};
    int32_t *d_status = reinterpret_cast<int32_t *>(sc);
    unsigned long long *d_badcode = reinterpret_cast<unsigned long long *>(sc + 8);
    Request *d_req = reinterpret_cast<Request *>(sc + off_req);
    int32_t *d_out = reinterpret_cast<int32_t *>(sc + off_out);
    PSet *d_ps = reinterpret_cast<PSet *>(sc + off_ps);
    void *d_P = sc + off_P;
    float *d_dlo = fp32 ? reinterpret_cast<float *>(sc + off_dlo) : nullptr;   // as the allocating path
    double *d_stage = stage64 ? reinterpret_cast<double *>(sc + off_stage) : nullptr;
    float *d_split = any_long ? reinterpret_cast<float *>(sc + off_split) : nullptr;
    WorkItem *d_wi = reinterpret_cast<WorkItem *>(sc + off_wi);
    int32_t *d_wib = reinterpret_cast<int32_t *>(sc + off_wib);
    double *d_part = reinterpret_cast<double *>(sc + off_part);
    double *d_elpr_out = d_elpr ? d_elpr : reinterpret_cast<double *>(sc + off_elpr);
    cudaStream_t s = cx.stream;
    const size_t nbytes = (size_t)total_cols * (size_t)cx.nl;
    // status key = none, invalid-code slot = none, error flag of timed-out waits cleared
    ce = cudaMemsetAsync(d_status, 0x7f, sizeof(int32_t), s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(d_badcode, 0xff, sizeof(unsigned long long), s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(cx.derr, 0, sizeof(int), s);
    // the caller's leaf codes are checked on the device, as pcsf_batch_create checks an upload
    if (ce == cudaSuccess && nbytes) ce = launch_check_codes(d_leaves, nbytes, d_badcode, s);
    unsigned long long bad = ~0ull;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&bad, d_badcode, sizeof(bad), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return pcsf_internal_fail(e, PCSF_ECUDA, cudaGetErrorString(ce));
    if (bad != ~0ull)
        return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: a leaf code is above PCSF_MARGINALIZE (64)");
    ce = cudaMemcpyAsync(d_req, h_req, sizeof(Request) * nreq, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_out, h_out, sizeof(int32_t) * nreq, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_ps, h_ps, sizeof(PSet), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess && nwi) ce = cudaMemcpyAsync(d_wi, h_wi, sizeof(WorkItem) * nwi, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_wib, h_wib, sizeof(int32_t) * (nreq + 1), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess && stage64) ce = launch_pform(true, d_ps, 1, cx.branch, cx.nbr, cx.m, d_stage, d_status, s);
    if (ce == cudaSuccess && any_long) ce = launch_split_ff(d_stage, d_split, nbr, s);
    if (ce == cudaSuccess && any_short) {
        if (fp32 && cx.pt64)   // FP64 formation rounded to FP32, as pcsf_lpr on a PCSF_PT_FP64 engine
            ce = launch_d2f_rows(d_stage, reinterpret_cast<float *>(d_P), nbr, cx.nbr, nullptr, cx.nl, s, d_dlo);
        else
            ce = launch_pform(!fp32, d_ps, 1, cx.branch, cx.nbr, cx.m, d_P, d_status, s, false, nullptr, 0, d_dlo);
    }
    PruneArgs pa{};
    pa.req = d_req;
    pa.leaves = d_leaves;
    pa.sched = cx.sched;
    pa.n_internal = cx.n_internal;
    pa.nl = cx.nl;
    pa.nbr = cx.nbr;
    pa.nslots = cx.nslots;
    pa.m = cx.m;
    pa.tile = cx.simt_tile;
    if (ce == cudaSuccess && nws) {
        pa.wi = d_wi;
        pa.nwi = nws;
        pa.Pbuf = d_P;
        pa.partials = d_part;
        pa.dither = fp32;     // as pcsf_lpr, so both give the same values
        pa.dlo = d_dlo;
        ce = launch_prune(fp32 ? PCSF_PREC_FP32 : PCSF_PREC_FP64, cx.comp, pa, s, std::min(cx.prune_grid, nws));
    }
    if (ce == cudaSuccess && nwi > nws) {
        pa.wi = d_wi + nws;
        pa.nwi = nwi - nws;
        pa.Pbuf = d_split;
        pa.partials = d_part + 2 * (size_t)nws;
        pa.dither = 0;
        pa.dlo = nullptr;
        ce = launch_prune_ff(pa, s, std::min(cx.ff_grid, nwi - nws));
    }
    if (ce == cudaSuccess) ce = launch_reduce(d_part, d_wib, nreq, d_lpr, d_elpr_out, s, d_out);
    int32_t key = STATUS_NONE;
    int herr = 0;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&key, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&herr, cx.derr, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return pcsf_internal_fail(e, PCSF_ECUDA, cudaGetErrorString(ce));
    if (herr) return pcsf_internal_fail(e, PCSF_ECUDA, "pcsf_lpr_noalloc: a device wait timed out");
    if (key >= 0 && key < 0x7f000000) return pcsf_internal_fail(e, key & 15, "pcsf_lpr_noalloc: P(t) formation failed");
    return PCSF_OK;
}
