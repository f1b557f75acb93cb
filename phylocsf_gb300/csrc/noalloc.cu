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
// is looked up once per device with cudaGetSymbolAddress (on the first call on
// that device, with that device current).  That first call should therefore
// come before any stream capture.  All calls share the one area and it keeps
// the previous call's contents: the parts that must start at zero are cleared
// on every call, and calls whose work overlaps on the GPU (from several host
// threads or engines on one device) race on it -- serialise them.  The host
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

static void *g_scratch_ptr[NOALLOC_MAX_DEVICES];
static std::once_flag g_scratch_once[NOALLOC_MAX_DEVICES];
static cudaError_t g_scratch_err[NOALLOC_MAX_DEVICES];

// Device address of the scratch array on `device` (which must be current).
static cudaError_t scratch_on(int device, unsigned char **out)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::call_once(g_scratch_once[device], [device] {
        g_scratch_err[device] = cudaGetSymbolAddress(&g_scratch_ptr[device], g_noalloc_scratch);
    });
    *out = reinterpret_cast<unsigned char *>(g_scratch_ptr[device]);
    return g_scratch_err[device];
}

}  // namespace pcsf

using namespace pcsf;

// Engine internals needed here (defined in engine.cpp).
int pcsf_internal_noalloc_ctx(pcsf_engine *e, int *device, cudaStream_t *stream, int *prec, int *compensated, int *nl,
                              int *nbr, const double **branch, const SchedNode **sched, int *n_internal, int *nslots,
                              DevModels *m, int *sm_count, int *prune_grid, int **derr);
int pcsf_internal_fail(pcsf_engine *e, int code, const char *msg);

extern "C" int pcsf_lpr_noalloc(pcsf_engine *e, int32_t model, double rho, int32_t n_regions,
                                const int64_t *col_offsets, const uint8_t *d_leaves, double *d_lpr, double *d_elpr)
{
    if (!e) return PCSF_EINVAL;
    int device, prec, comp, nl, nbr, nint, nslots, smc, pgrid;
    cudaStream_t s;
    const double *branch;
    const SchedNode *sched;
    DevModels m;
    int *derr;
    pcsf_internal_noalloc_ctx(e, &device, &s, &prec, &comp, &nl, &nbr, &branch, &sched, &nint, &nslots, &m, &smc,
                              &pgrid, &derr);
    if (cudaSetDevice(device) != cudaSuccess) return pcsf_internal_fail(e, PCSF_ECUDA, "pcsf_lpr_noalloc: cudaSetDevice");
    if (model < 0 || model > 1) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: model must be 0 or 1");
    if (!(rho > 0.0) || !std::isfinite(rho)) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: rho must be > 0");
    if (n_regions < 0 || (n_regions > 0 && (!col_offsets || !d_lpr)))
        return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: null argument");
    if (n_regions > NOALLOC_MAX_REGIONS)
        return pcsf_internal_fail(e, PCSF_ERANGE, "pcsf_lpr_noalloc: more than 32768 regions in one call");
    if (n_regions == 0) return PCSF_OK;
    if (col_offsets[0] != 0) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: col_offsets[0] must be 0");
    // every returned likelihood comes from the SIMT kernels (compensated FP32 on
    // reduced-precision engines), as pcsf_lpr does
    const int TC = simt_tile_cols(prec, nslots);
    const size_t es = prec == PCSF_PREC_FP64 ? 8 : 4;
    // scratch map: [status key][requests][P set][diag(E) low parts][work items][wi_begin][partials]
    const size_t off_req = 256;
    const size_t off_ps = off_req + ((sizeof(Request) * n_regions + sizeof(PSet) + 255) & ~size_t(255));
    const size_t off_P = off_ps + 256;
    const size_t pbytes = (size_t)nbr * K2 * es;
    const size_t off_dlo = off_P + ((pbytes + 255) & ~size_t(255));
    const bool fp32 = prec != PCSF_PREC_FP64;
    const size_t off_wi = off_dlo + (fp32 ? (((size_t)nbr * K * sizeof(float) + 255) & ~size_t(255)) : 0);
    int nwi = 0;
    for (int r = 0; r < n_regions; r++) {
        const int64_t c0 = col_offsets[r], c1 = col_offsets[r + 1];
        if (c1 < c0) return pcsf_internal_fail(e, PCSF_EINVAL, "pcsf_lpr_noalloc: col_offsets not non-decreasing");
        h_req[r] = Request{r, model, 0, (uint32_t)c0, rho};
        h_wib[r] = nwi;
        for (int64_t c = c0; c < c1; c += TC) {
            if (nwi >= NOALLOC_MAX_WORK)
                return pcsf_internal_fail(e, PCSF_ERANGE, "pcsf_lpr_noalloc: more than 131072 column tiles in one call");
            h_wi[nwi++] = WorkItem{r, (int32_t)std::min<int64_t>(TC, c1 - c), c};
        }
    }
    h_wib[n_regions] = nwi;
    const size_t off_wib = off_wi + ((sizeof(WorkItem) * (size_t)nwi + 255) & ~size_t(255));
    const size_t off_part = off_wib + ((sizeof(int32_t) * (size_t)(n_regions + 1) + 255) & ~size_t(255));
    const size_t need = off_part + sizeof(double) * 2 * (size_t)std::max(nwi, 1);
    if (need > NOALLOC_BYTES)
        return pcsf_internal_fail(e, PCSF_ERANGE, "pcsf_lpr_noalloc: batch needs more than the 24 MiB static scratch area");
    unsigned char *sc = nullptr;
    cudaError_t ce = scratch_on(device, &sc);
    if (ce != cudaSuccess) return pcsf_internal_fail(e, PCSF_ECUDA, "pcsf_lpr_noalloc: cudaGetSymbolAddress failed");
    h_ps[0] = PSet{model, 0, rho};
    int32_t *d_status = reinterpret_cast<int32_t *>(sc);
    Request *d_req = reinterpret_cast<Request *>(sc + off_req);
    PSet *d_ps = reinterpret_cast<PSet *>(sc + off_ps);
    void *d_P = sc + off_P;
    float *d_dlo = fp32 ? reinterpret_cast<float *>(sc + off_dlo) : nullptr;   // as the allocating path
    WorkItem *d_wi = reinterpret_cast<WorkItem *>(sc + off_wi);
    int32_t *d_wib = reinterpret_cast<int32_t *>(sc + off_wib);
    double *d_part = reinterpret_cast<double *>(sc + off_part);
    double *d_elpr_out = d_elpr ? d_elpr : d_part + 2 * (size_t)nwi;   // unused tail when no elpr output
    if (!d_elpr && need + sizeof(double) * n_regions > NOALLOC_BYTES)
        return pcsf_internal_fail(e, PCSF_ERANGE, "pcsf_lpr_noalloc: batch needs more than the 24 MiB static scratch area");
    ce = cudaMemsetAsync(d_status, 0x7f, sizeof(int32_t), s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_req, h_req, sizeof(Request) * n_regions, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_ps, h_ps, sizeof(PSet), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess && nwi) ce = cudaMemcpyAsync(d_wi, h_wi, sizeof(WorkItem) * nwi, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_wib, h_wib, sizeof(int32_t) * (n_regions + 1), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess)
        ce = launch_pform(prec == PCSF_PREC_FP64, d_ps, 1, branch, nbr, m, d_P, d_status, s, false, nullptr, 0, d_dlo);
    if (ce == cudaSuccess && nwi) {
        PruneArgs pa{};
        pa.wi = d_wi;
        pa.nwi = nwi;
        pa.req = d_req;
        pa.leaves = d_leaves;
        pa.Pbuf = d_P;
        pa.sched = sched;
        pa.n_internal = nint;
        pa.nl = nl;
        pa.nbr = nbr;
        pa.nslots = nslots;
        pa.m = m;
        pa.partials = d_part;
        pa.dither = prec != PCSF_PREC_FP64;     // as pcsf_lpr, so both give the same values
        pa.dlo = d_dlo;
        const bool tcprec = prec == PCSF_PREC_TF32X3 || prec == PCSF_PREC_TF32;
        ce = launch_prune(prec == PCSF_PREC_FP64 ? PCSF_PREC_FP64 : PCSF_PREC_FP32, (comp == 0 && tcprec) ? 1 : comp, pa,
                          s, std::min(pgrid, nwi));
    }
    if (ce == cudaSuccess) ce = launch_reduce(d_part, d_wib, n_regions, d_lpr, d_elpr_out, s);
    int32_t key = STATUS_NONE;
    int herr = 0;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&key, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return pcsf_internal_fail(e, PCSF_ECUDA, cudaGetErrorString(ce));
    if (herr) return pcsf_internal_fail(e, PCSF_ECUDA, "pcsf_lpr_noalloc: a tensor-core wait timed out");
    if (key >= 0 && key < 0x7f000000) return pcsf_internal_fail(e, key & 15, "pcsf_lpr_noalloc: P(t) formation failed");
    return PCSF_OK;
}
