// The network pass without device allocation (ann_network_noalloc).
#include "context.hpp"

// ---------------------------------------------------------------- no-allocation network pass
// ann_network_noalloc runs the network stage (per-type atom lists, then the per-element networks)
// on symmetry functions the caller already holds on the device, and allocates no device memory:
// its scratch (status word and per-type lists) is carved from one static device array of this
// file. It serves callers that must not allocate during a step, such as an MD engine or plugin
// host that reserves its device memory up front and runs every step inside that reservation
// (cudaMalloc / cudaFree synchronise the device and can fail mid-run under memory pressure).
// Every call on a device shares the array, so calls that overlap in time (other host threads,
// other contexts, other streams) race on it and must be serialised by the caller.
namespace {
constexpr size_t NOALLOC_MAX_ATOMS = ANN_NOALLOC_MAX_ATOMS;
constexpr size_t NA_STATUS = 0;                                            // int32[8]
constexpr size_t NA_TSTART = 256;                                          // int32[MAXT+1]
constexpr size_t NA_TCOUNT = 512;                                          // int32[MAXT+1+natoms]
constexpr size_t NA_TLIST = NA_TCOUNT + ((4 * (MAXT + 1 + NOALLOC_MAX_ATOMS) + 255) / 256) * 256;  // int32[natoms]
constexpr size_t NA_BYTES = NA_TLIST + 4 * NOALLOC_MAX_ATOMS;
static_assert(NA_BYTES <= ANN_NOALLOC_SCRATCH_BYTES, "no-allocation scratch layout exceeds the static array");
}  // namespace
static __device__ __align__(256) unsigned char g_noalloc_scratch[ANN_NOALLOC_SCRATCH_BYTES];

// device address of the scratch array in the current device's context. The host-side name
// g_noalloc_scratch is only a stand-in, never a device address. The address is looked up on every
// call (a host query that allocates nothing), so a context that the application destroyed and
// re-created (cudaDeviceReset) never leaves a stale address behind
static unsigned char* noalloc_scratch() {
    unsigned char* p = nullptr;
    ck(cudaGetSymbolAddress((void**)&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-allocation scratch)");
    return p;
}

extern "C" {
int ann_network_noalloc(ann_ctx* c, int32_t natoms, const int32_t* type_dev, const void* G_dev, double* Eatom_dev, void* dEdG_dev,
                        int32_t precision) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        if (!c->have_pot) throw ann_error(ANN_ERR_STATE, "no potential loaded");
        if (precision != ANN_FP64 && precision != ANN_MIXED) throw ann_error(ANN_ERR_ARG, "invalid precision");
        if (natoms < 0) throw ann_error(ANN_ERR_ARG, "natoms must be >= 0");
        if ((size_t)natoms > NOALLOC_MAX_ATOMS)
            throw ann_error(ANN_ERR_CAPACITY, "ann_network_noalloc takes at most " + std::to_string(NOALLOC_MAX_ATOMS) + " atoms per call (got " +
                                                  std::to_string(natoms) + "); use ann_compute or split the call");
        if (natoms > 0 && (!type_dev || !G_dev || !Eatom_dev || !dEdG_dev)) throw ann_error(ANN_ERR_ARG, "NULL device pointer");
        set_device(c);
        const bool fp64 = precision == ANN_FP64;
        const bool tc = !fp64 && use_tc(c);
        const DevPot& pot = c->plan.pot;
        if (!tc && mlp_smem_bytes(pot, fp64, false) + 1024 > (size_t)c->max_smem)
            throw ann_error(ANN_ERR_UNSUPPORTED, "networks too wide for the shared-memory network kernel");
        unsigned char* s = noalloc_scratch();
        int32_t* status = reinterpret_cast<int32_t*>(s + NA_STATUS);
        int32_t* tstart = reinterpret_cast<int32_t*>(s + NA_TSTART);
        int32_t* tcount = reinterpret_cast<int32_t*>(s + NA_TCOUNT);
        int32_t* tlist = reinterpret_cast<int32_t*>(s + NA_TLIST);
        cudaStream_t st = c->stream;
        // the status word starts at zero; launch_type_lists clears the per-type counters itself
        ck(cudaMemsetAsync(status, 0, 32, st), "clear no-allocation status");
        const int64_t before = g_launch_counter;
        launch_type_lists(natoms, c->pot.ntypes(), type_dev, tcount, tstart, tlist, status, st);
        if (tc) {
            for (int ty = 0; ty < c->pot.ntypes(); ++ty) {
                TcArgs ta{};
                ta.natoms = natoms; ta.imax = pot.imax; ta.type = ty;
                ta.tstart = tstart; ta.tlist = tlist;
                ta.G = static_cast<const float*>(G_dev); ta.dEdG = static_cast<float*>(dEdG_dev); ta.Eatom = Eatom_dev;
                ta.image = c->tcimg.as<uint8_t>(); ta.status = status; ta.wait_polls = c->wait_polls;
                launch_mlp_tc(c->tc.t[ty], ta, natoms / c->pot.ntypes(), c->tune_tc[ty] ? c->tune_tc[ty] : c->opt.tc_groups, c->tc.smem_bytes(ty), c->nsm, st);
            }
        } else if (fp64) {
            MlpArgs<double> m{};
            m.natoms = natoms; m.ntypes = c->pot.ntypes(); m.imax = pot.imax; m.tstart = tstart; m.tlist = tlist;
            m.G = static_cast<const double*>(G_dev); m.dEdG = static_cast<double*>(dEdG_dev); m.Eatom = Eatom_dev;
            m.prm = c->pd.view();
            launch_mlp_forward_backward<double>(pot, m, st);
        } else {
            MlpArgs<float> m{};
            m.natoms = natoms; m.ntypes = c->pot.ntypes(); m.imax = pot.imax; m.tstart = tstart; m.tlist = tlist;
            m.G = static_cast<const float*>(G_dev); m.dEdG = static_cast<float*>(dEdG_dev); m.Eatom = Eatom_dev;
            m.prm = c->pf.view();
            launch_mlp_forward_backward<float>(pot, m, st);
        }
        c->kernels += g_launch_counter - before;
        ck(cudaGetLastError(), "no-allocation network launch");
        int32_t hst[8];
        ck(cudaMemcpyAsync(hst, status, sizeof(hst), cudaMemcpyDeviceToHost, st), "D2H no-allocation status");
        ck(cudaStreamSynchronize(st), "synchronize");
        if (hst[0] & ST_BAD_TYPE) throw ann_error(ANN_ERR_ARG, "type index out of range");
        if (hst[0] & ST_TIMEOUT) throw ann_error(ANN_ERR_TIMEOUT, "a bounded device wait gave up");
        if (hst[0]) throw ann_error(ANN_ERR_CUDA, "unknown device status " + std::to_string(hst[0]));
    })
}
}  // extern "C"
