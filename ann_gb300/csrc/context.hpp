// Private to libann_gpu: the context behind the C ABI (ann_ctx) and what its translation units
// share. context.cu holds creation, potentials, batches and inspection; list.cu the caller's
// neighbour lists; train_host.cu input statistics, training and the optimiser; md_host.cu molecular
// dynamics; noalloc.cu the network pass without allocation.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ann_gpu.h"
#include "kernels.hpp"
#include "mlp_tc.hpp"
#include "plan_build.hpp"
#include "potential.hpp"

namespace ann {
// training loss / adjoint seeds (train.cu)
void launch_train_loss(int nstruc, int natoms, const int32_t* off, const int32_t* sid, const double* Es, const double* Fout,
                       const double* Eref, const double* Fref, double wE, double wF, int lossf, int norm, double delta, double* loss3,
                       double* ce, void* lam, bool fp64, cudaStream_t st);
void launch_md_kick_drift(int natoms, double* pos, double* vel, const void* F, bool fp64, const double* minv, const int32_t* type,
                          double dt, const double* R, const double* Ri, double* disp_ref, int32_t* maxdisp_flag, double half_skin2,
                          int stage, cudaStream_t st);
void launch_md_ke(int natoms, const double* vel, const double* mass, const int32_t* type, double* ke, cudaStream_t st);
// optimiser and parameter refresh (optim.cu)
void launch_param_refresh(int64_t n, const double* p, const int32_t* map, double* w64, double* wt64, double* b64, float* w32, float* wt32,
                          float* b32, uint8_t* img, cudaStream_t st);
void configure_kernels();
}

using namespace ann;

// every (re)allocation of a device buffer bumps this counter; captured graphs record it and are
// recaptured when it moved (a graph holds raw buffer pointers)
extern std::atomic<uint64_t> g_alloc_gen;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void ensure(size_t b) {
        if (b <= bytes && p) return;
        ++g_alloc_gen;
        if (p) cudaFree(p);
        p = nullptr; bytes = 0;
        const size_t want = std::max<size_t>(b, 256);
        const cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) { p = nullptr; throw ann_error(ANN_ERR_CUDA, std::string("cudaMalloc(") + std::to_string(want) + "): " + cudaGetErrorString(e)); }
        bytes = want;
    }
    void release() { if (p) cudaFree(p); p = nullptr; bytes = 0; }
    template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

template <typename real>
struct ParamSet {
    DevBuf rs, reta, aeta, zeta, alam, agrp, slot2ref, w, wt, b, inpw, inpb;
    DevParams<real> view() const {
        DevParams<real> d;
        d.rs = rs.as<real>(); d.reta = reta.as<real>(); d.aeta = aeta.as<real>(); d.zeta = zeta.as<real>(); d.alam = alam.as<real>();
        d.agrp = agrp.as<int32_t>(); d.slot2ref = slot2ref.as<int32_t>();
        d.w = w.as<real>(); d.wt = wt.as<real>(); d.b = b.as<real>(); d.inpw = inpw.as<real>(); d.inpb = inpb.as<real>();
        return d;
    }
    void release() { for (DevBuf* x : {&rs, &reta, &aeta, &zeta, &alam, &agrp, &slot2ref, &w, &wt, &b, &inpw, &inpb}) x->release(); }
};

template <typename real> DevParams<real> params_of(ParamSet<float>& f, ParamSet<double>& d);
template <> inline DevParams<float> params_of<float>(ParamSet<float>& f, ParamSet<double>&) { return f.view(); }
template <> inline DevParams<double> params_of<double>(ParamSet<float>&, ParamSet<double>& d) { return d.view(); }

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw ann_error(ANN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// the three forms of the E+F kernel sequence (graph slots of ann_ctx::gexec)
enum { SEQ_BUILD = 0, SEQ_REFRESH = 1, SEQ_STAGED = 2 };

struct GraphKey {
    int S, N, cap, prec, forces, nbins, nchunks;
    int md;         // MD mode: list cutoff rc + skin, refreshed between rebuilds
    uint64_t gen;   // g_alloc_gen at capture
    int flags;      // bit 0: structures binned one block each (nbr_local_binning of the largest
                    // structure); bit 1: per-structure sums in one launch (no empty structure)
    bool operator==(const GraphKey& o) const {
        return S == o.S && N == o.N && cap == o.cap && prec == o.prec && forces == o.forces && nbins == o.nbins && nchunks == o.nchunks &&
               md == o.md && gen == o.gen && flags == o.flags;
    }
};

struct ann_ctx {
    ann_options opt;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;                 // fork / join branch of the E+F sequence
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_net_fork = nullptr, ev_net_join = nullptr;   // the per-type network launches on two streams
    std::string err;
    bool have_pot = false;
    Potential pot;
    PlanHost plan;
    TcPlan tc;                      // tensor-core network images (MIXED precision)
    TcTrainLayout tct[MAXT];        // the training kernel's layout per type
    bool tct_ok = false;            // every type fits the tensor-core training kernel
    DevBuf tcimg;
    // packed FP64 parameters on the device and where each one is copied to
    DevBuf p64, pmap;
    bool params_dev_newer = false;  // an optimiser step changed p64 after the host copy
    // optimiser state (opt::algo, src/opt/algo.cpp): s0 / s1 / s2 per parameter, the previous
    // gradient, and the CG reduction
    DevBuf opt_s0, opt_s1, opt_s2, opt_gold, opt_part;
    bool opt_ready = false, have_grad = false;
    int opt_algo = 7;                         // ADAM
    int64_t opt_t = 0;
    double opt_lr = 0, opt_b1 = 0.9, opt_b2 = 0.999, opt_eps = 0, opt_eta = 0, opt_w = 0;
    double opt_b1i = 0, opt_b2i = 0;          // beta^t, kept as running products (opt/algo.cpp:275-295)
    double opt_gamma = 0;                     // the step size after the decay schedule
    int opt_decay = 1, opt_period = 1, opt_reg = 4;      // Decay CONST, Regularization NONE
    double opt_alpha = 0, opt_reg_eta = 0;
    double last_loss = 0, prev_loss = 0;      // training loss of the last forward pass / of the previous step (RPROP)
    ParamSet<float> pf;
    ParamSet<double> pd;
    DevBuf poff;
    // batch
    int S = 0, N = 0;
    int max_nat = 0;                // atoms of the largest structure of the staged batch
    uint64_t tables_gen = ~0ull;    // g_alloc_gen when the offset tables and sid were last uploaded
    bool red_fused = false;         // every structure has atoms: per-structure sums in one launch
    int nn_seen = 0;                // longest neighbour row of the batches computed so far (list cutoff rc)
    DevBuf rarrive;                 // [S] per-structure chunk arrivals of that launch (zero between launches)
    bool have_batch = false;
    std::vector<int32_t> off_h, rchunk_h, rschunk_h, tables_h;
    DevBuf tables, cell, pos, type, sid, rpartial;
    const int32_t* off_d = nullptr;        // device offsets [S+1] (inside tables)
    const int32_t* rchunk_d = nullptr;     // reduction chunks [3 * nchunks] (inside tables)
    const int32_t* rschunk_d = nullptr;    // first chunk of each structure [S+1] (inside tables)
    // neighbour list
    int cap = 0, nbins_cap = 0;
    DevBuf geo, pos4, abin, abc, am, aslot, bcount, bstart, bidx, bm, bpos4, bposd, nn, ntc, nj, nimg, nr, scan_tmp, counter, status;
    // per atom / structure
    DevBuf G, dEdG, Eatom, F, W, Es, Ws, Fout, tcount, tstart, tlist;
    int last_prec = -1;
    bool have_results = false, have_forces = false;
    // graphs
    // graphs of the E+F sequence: [SEQ_BUILD] with the list build, [SEQ_REFRESH] with the Verlet-list
    // refresh (MD), [SEQ_STAGED] from the networks on (neighbour rows and G of the staged training batch)
    cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
    GraphKey gkey[3] = {{-1, -1, -1, -1, -1, -1, -1, -1, 0, -1}, {-1, -1, -1, -1, -1, -1, -1, -1, 0, -1}, {-1, -1, -1, -1, -1, -1, -1, -1, 0, -1}};
    // training
    DevBuf Eref, Fref, loss3, ce, lam, U, grad, gpart;   // gpart: per-block gradient sums of the training pass
    bool have_train = false;
    int train_prec = 0;
    // the batch of the last ann_train_forward with its neighbour rows, type lists and symmetry
    // functions (in train_staged_prec) still on the device, for ann_train_forward_staged; cleared by
    // any other batch, E+F sequence or potential load
    bool train_staged = false;
    int train_staged_prec = 0;
    double train_wE = 0, train_wF = 0;
    int train_loss = ANN_LOSS_MSE, train_norm = ANN_NORM_LINEAR;   // energy term (ann_train_set_loss)
    double train_delta = 1.0;
    // MD
    bool md_ready = false;
    int md_prec = 0;
    double md_dt = 0, md_skin = 0;
    DevBuf vel, minv, mass, disp_ref, mdflag, ke;
    std::vector<double> md_mass_t;
    double md_R[9], md_Ri[9];
    DevBuf md_R_d, md_Ri_d;
    int md_rebuilds = 0;
    // a caller's neighbour list (ann_compute_list): inputs, rows and results, apart from the batch
    DevBuf lx, lxh, lxl, ltype, lilist, lnoff, lneigh, lrtype, lnn, lntc, lnj, lnr, lG, ldEdG, lEatom, lF, lW, lFout, ltcount, ltstart, ltlist,
        ltables, lpartial, lEs, lWs;
    int list_hint = 0;              // longest row within rc seen so far
    bool list_staged = false, list_have_ilist = false;   // a list on the device that ANN_LIST_KEEP may reuse
    int list_inum = 0, list_nall = 0, list_maxnn = 0;
    // input statistics of a training set (ann_stats_*): accumulators [T][6][imax] and counts [T]
    DevBuf st_acc, st_n, st_part, st_pcount;
    bool st_ready = false;
    int st_T = 0, st_imax = 0;
    // instrumentation
    int64_t kernels = 0;            // kernels launched (graph replays add graph_kernels)
    int64_t graph_kernels[3] = {0, 0, 0};
    bool profile = false;
    bool debug = false;             // synchronise and check after every phase (ANN_DEBUG=1)
    int max_smem = 48 * 1024;       // opt-in shared memory per block of the device
    int nsm = 1;                    // streaming multiprocessors of the device (persistent grids)
    int32_t wait_polls = 0;         // kernel argument of ann_set_wait_limit: 0 built-in bounds, k > 0 at most k - 1 polls
    int32_t* status_h = nullptr;    // page-locked copy of the status word
    // launch shapes chosen by ann_autotune / ann_set_tuning (0: the built-in rule)
    int32_t tune_tc[MAXT] = {0, 0, 0, 0};
    int32_t tune_bp = 0, tune_nbr = 0;
    cudaEvent_t ev[16] = {};
};

namespace ann { extern thread_local int64_t g_launch_counter; }

// error reporting: the context's and the thread-wide last error; every C ABI body runs in ANN_TRY
int fail(ann_ctx* c, int code, const std::string& m);
#define ANN_TRY(ctx, ...)                                                                 \
    try { __VA_ARGS__; return ANN_OK; }                                                   \
    catch (ann_error& e) { return fail(ctx, e.code, e.what()); }                          \
    catch (std::exception& e) { return fail(ctx, ANN_ERR_ARG, e.what()); }

void set_device(ann_ctx* c);
// potential and parameters
void rebuild_plan(ann_ctx* c);
void sync_params_from_device(ann_ctx* c);
// batches and the E+F sequence
void leave_md(ann_ctx* c);
void upload_batch(ann_ctx* c, int nstruc, const int64_t* offs, const double* posn, const int32_t* type, const double* cell, bool device_src);
void run_batch(ann_ctx* c, int prec, bool forces, bool build_list = true);
// the E+F sequence from the networks on, over the neighbour rows, type lists and symmetry
// functions that the last ann_train_forward left on the device (c->train_staged)
void run_staged(ann_ctx* c, int prec);
void finish_batch(ann_ctx* c);
// the longest neighbour row of a finished batch (status word 3), for the capacity of later batches
inline void note_rows(ann_ctx* c, const int32_t* st) { if (!c->md_ready) c->nn_seen = std::max(c->nn_seen, (int)st[3]); }
int32_t* status_host(ann_ctx* c);
// drops the captured graphs (launch shapes changed)
void drop_graphs(ann_ctx* c);

template <typename real>
inline BpArgs<real> bp_args(ann_ctx* c) {
    BpArgs<real> b{};
    b.natoms = c->N; b.ntypes = c->pot.ntypes(); b.cap = c->cap; b.newton_untranslated = (c->opt.newton == ANN_NEWTON_UNTRANSLATED);
    b.type = c->type.as<int32_t>(); b.nn = c->nn.as<int32_t>(); b.ntc = c->ntc.as<int32_t>(); b.nj = c->nj.as<int32_t>(); b.nimg = c->nimg.as<int32_t>();
    b.nr = c->nr.p; b.G = c->G.as<real>(); b.dEdG = c->dEdG.as<real>(); b.F = c->F.as<real>(); b.W = c->W.as<real>();
    b.lam = c->lam.as<real>(); b.U = c->U.as<real>();
    b.counter = c->counter.as<uint32_t>(); b.status = c->status.as<int32_t>();
    b.grid_per_sm = c->tune_bp;
    b.nsm = c->nsm;
    b.wait_polls = c->wait_polls;
    return b;
}

// the MIXED network pass runs on the tensor cores unless the SIMT kernels are asked for
inline bool use_tc(const ann_ctx* c) { return c->opt.mlp_backend != 1 && c->tc.ok; }

// the network stage: per-atom energies and dE/dG of natoms atoms grouped by type (tstart/tlist)
template <typename real>
inline void enqueue_networks(ann_ctx* c, int natoms, DevBuf& G, DevBuf& dEdG, DevBuf& Eatom, DevBuf& tstart, DevBuf& tlist,
                             const DevParams<real>& prm) {
    const DevPot& pot = c->plan.pot;
    if (!std::is_same<real, double>::value && use_tc(c)) {
        // one launch per type; outside the phase-timed and debug modes the odd types run on the side
        // stream, so that the types' tiles share the SMs (a small batch leaves most SMs idle in each
        // launch). CTAs of different types may then share an SM: every launch asks for the shared
        // memory that admits at most 512 / (widest TMEM allocation) CTAs per SM, so that co-resident
        // CTAs never need more than the SM's 512 tensor-memory columns together.
        const int T = c->pot.ntypes();
        const bool fork = T > 1 && !c->profile && !c->debug;
        int cmax = 32;
        for (int ty = 0; ty < T; ++ty) cmax = std::max(cmax, (int)c->tc.t[ty].tmem_cols);
        if (fork) {
            ck(cudaEventRecord(c->ev_net_fork, c->stream), "event record");
            ck(cudaStreamWaitEvent(c->side, c->ev_net_fork, 0), "stream wait");
        }
        for (int ty = 0; ty < T; ++ty) {
            TcArgs ta{};
            ta.natoms = natoms; ta.imax = pot.imax; ta.type = ty;
            ta.tstart = tstart.as<int32_t>(); ta.tlist = tlist.as<int32_t>();
            ta.G = G.as<float>(); ta.dEdG = dEdG.as<float>(); ta.Eatom = Eatom.as<double>();
            ta.image = c->tcimg.as<uint8_t>(); ta.status = c->status.as<int32_t>(); ta.wait_polls = c->wait_polls;
            size_t smem = c->tc.smem_bytes(ty);
            if (fork) smem = std::max(smem, (size_t)c->tc.smem_per_sm / (size_t)(512 / cmax + 1) + 1);
            launch_mlp_tc(c->tc.t[ty], ta, natoms / T, c->tune_tc[ty] ? c->tune_tc[ty] : c->opt.tc_groups, smem, c->nsm,
                          (fork && (ty & 1)) ? c->side : c->stream);
        }
        if (fork) {
            ck(cudaEventRecord(c->ev_net_join, c->side), "event record");
            ck(cudaStreamWaitEvent(c->stream, c->ev_net_join, 0), "stream wait");
        }
    } else {
        MlpArgs<real> m{};
        m.natoms = natoms; m.ntypes = c->pot.ntypes(); m.imax = pot.imax;
        m.tstart = tstart.as<int32_t>(); m.tlist = tlist.as<int32_t>();
        m.G = G.as<real>(); m.dEdG = dEdG.as<real>(); m.Eatom = Eatom.as<double>();
        m.prm = prm;
        launch_mlp_forward_backward<real>(pot, m, c->stream);
    }
}
