// ann_ctx: device buffers, the per-batch kernel sequence, CUDA-graph capture, and the extern "C"
// entry points of include/ann_gpu.h. No C++ exception crosses the C boundary.
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
                       const double* Eref, const double* Fref, double wE, double wF, double* loss3, double* ce, void* lam,
                       bool fp64, cudaStream_t st);
void launch_md_kick_drift(int natoms, double* pos, double* vel, const void* F, bool fp64, const double* minv, const int32_t* type,
                          double dt, const double* R, const double* Ri, double* disp_ref, int32_t* maxdisp_flag, double half_skin2,
                          int stage, cudaStream_t st);
void launch_md_ke(int natoms, const double* vel, const double* mass, const int32_t* type, double* ke, cudaStream_t st);
// optimiser and parameter refresh (optim.cu)
void launch_adam(int64_t n, const double* g, double scale, double* m, double* v, double* p, double lr, double b1, double b2, double b1ii,
                 double b2ii, double eps, cudaStream_t st);
void launch_param_refresh(int64_t n, const double* p, const int32_t* map, double* w64, double* wt64, double* b64, float* w32, float* wt32,
                          float* b32, uint8_t* img, cudaStream_t st);
void configure_kernels();
}

using namespace ann;

static std::mutex g_err_mu;
static std::string g_err;

// every (re)allocation of a device buffer bumps this counter; captured graphs record it and are
// recaptured when it moved (a graph holds raw buffer pointers)
static std::atomic<uint64_t> g_alloc_gen{0};

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

template <typename real> static DevParams<real> params_of(ParamSet<float>& f, ParamSet<double>& d);
template <> DevParams<float> params_of<float>(ParamSet<float>& f, ParamSet<double>&) { return f.view(); }
template <> DevParams<double> params_of<double>(ParamSet<float>&, ParamSet<double>& d) { return d.view(); }

static void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw ann_error(ANN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename real>
static void upload_vec(DevBuf& b, const std::vector<double>& v, cudaStream_t st) {
    std::vector<real> h(v.begin(), v.end());
    b.ensure(h.size() * sizeof(real));
    ck(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(real), cudaMemcpyHostToDevice, st), "upload params");
    ck(cudaStreamSynchronize(st), "upload params");
}
static void upload_ints(DevBuf& b, const std::vector<int>& v, cudaStream_t st) {
    b.ensure(v.size() * sizeof(int32_t));
    ck(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st), "upload params");
    ck(cudaStreamSynchronize(st), "upload params");
}

struct GraphKey {
    int S, N, cap, prec, forces, nbins, nchunks;
    uint64_t gen;   // g_alloc_gen at capture
    bool operator==(const GraphKey& o) const {
        return S == o.S && N == o.N && cap == o.cap && prec == o.prec && forces == o.forces && nbins == o.nbins && nchunks == o.nchunks &&
               gen == o.gen;
    }
};

struct ann_ctx {
    ann_options opt;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;                 // fork / join branch of the E+F sequence
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string err;
    bool have_pot = false;
    Potential pot;
    PlanHost plan;
    TcPlan tc;                      // tensor-core network images (MIXED precision)
    DevBuf tcimg;
    // packed FP64 parameters on the device and where each one is copied to
    DevBuf p64, pmap;
    bool params_dev_newer = false;  // an optimiser step changed p64 after the host copy
    // Adam state (NN::ADAM, opt/algo.cpp:272-296)
    DevBuf adam_m, adam_v;
    bool adam_ready = false, have_grad = false;
    int64_t adam_t = 0;
    double adam_lr = 0, adam_b1 = 0, adam_b2 = 0, adam_eps = 0;
    ParamSet<float> pf;
    ParamSet<double> pd;
    DevBuf poff;
    // batch
    int S = 0, N = 0;
    bool have_batch = false;
    std::vector<int32_t> off_h, rchunk_h, rschunk_h, tables_h;
    DevBuf tables, cell, pos, type, sid, rpartial;
    const int32_t* off_d = nullptr;        // device offsets [S+1] (inside tables)
    const int32_t* rchunk_d = nullptr;     // reduction chunks [3 * nchunks] (inside tables)
    const int32_t* rschunk_d = nullptr;    // first chunk of each structure [S+1] (inside tables)
    // neighbour list
    int cap = 0, nbins_cap = 0;
    DevBuf geo, pos4, abin, abc, am, aslot, bcount, bstart, bidx, bm, bpos4, bposd, nbins_total, nn, ntc, nj, nimg, nr, scan_tmp, counter, status;
    // per atom / structure
    DevBuf G, dEdG, Eatom, F, W, Es, Ws, Fout, tcount, tstart, tlist;
    int last_prec = -1;
    bool have_results = false, have_forces = false;
    // graphs
    // graphs of the E+F sequence: [0] with the list build, [1] with the Verlet-list refresh (MD)
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    GraphKey gkey[2] = {{-1, -1, -1, -1, -1, -1, -1, 0}, {-1, -1, -1, -1, -1, -1, -1, 0}};
    // training
    DevBuf Eref, Fref, loss3, ce, lam, U, grad;
    bool have_train = false;
    int train_prec = 0;
    double train_wE = 0, train_wF = 0;
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
    DevBuf lx, ltype, lilist, lnoff, lneigh, lrtype, lnn, lntc, lnj, lnr, lG, ldEdG, lEatom, lF, lW, lFout, ltcount, ltstart, ltlist,
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
    int64_t graph_kernels[2] = {0, 0};
    bool profile = false;
    bool debug = false;             // synchronise and check after every phase (ANN_DEBUG=1)
    int max_smem = 48 * 1024;       // opt-in shared memory per block of the device
    int32_t* status_h = nullptr;    // page-locked copy of the status word
    cudaEvent_t ev[16] = {};
};

namespace ann { extern thread_local int64_t g_launch_counter; }

static int fail(ann_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    std::lock_guard<std::mutex> g(g_err_mu);
    g_err = m;
    return code;
}
#define ANN_TRY(ctx, ...)                                                                 \
    try { __VA_ARGS__; return ANN_OK; }                                                   \
    catch (ann_error& e) { return fail(ctx, e.code, e.what()); }                          \
    catch (std::exception& e) { return fail(ctx, ANN_ERR_ARG, e.what()); }

static void set_device(ann_ctx* c) { ck(cudaSetDevice(c->opt.device), "cudaSetDevice"); }

// ---------------------------------------------------------------- potential upload
template <typename real>
static void upload_params(ann_ctx* c, ParamSet<real>& P) {
    const PlanHost& h = c->plan;
    upload_vec<real>(P.rs, h.rs, c->stream); upload_vec<real>(P.reta, h.reta, c->stream);
    upload_vec<real>(P.aeta, h.aeta, c->stream); upload_vec<real>(P.zeta, h.zeta, c->stream); upload_vec<real>(P.alam, h.alam, c->stream);
    upload_ints(P.agrp, h.agrp, c->stream); upload_ints(P.slot2ref, h.slot2ref, c->stream);
    upload_vec<real>(P.w, h.w, c->stream); upload_vec<real>(P.wt, h.wt, c->stream); upload_vec<real>(P.b, h.b, c->stream);
    upload_vec<real>(P.inpw, h.inpw, c->stream); upload_vec<real>(P.inpb, h.inpb, c->stream);
}
static void reset_graph(ann_ctx* c) {
    for (int k = 0; k < 2; ++k) {
        if (c->gexec[k]) { cudaGraphExecDestroy(c->gexec[k]); c->gexec[k] = nullptr; }
        c->gkey[k] = GraphKey{-1, -1, -1, -1, -1, -1, -1, 0};
    }
}
static void rebuild_plan(ann_ctx* c) {
    build_plan(c->pot, c->plan);
    build_tc_plan(c->plan.pot, c->plan.w, c->plan.b, c->plan.inpw, c->plan.inpb, c->max_smem, c->tc);
    if (c->opt.mlp_backend == 2 && !c->tc.ok)
        throw ann_error(ANN_ERR_UNSUPPORTED, "the networks do not fit the tensor-core kernel (hidden layers 1..5, widths <= 256)");
    c->tcimg.ensure(c->tc.image.size());
    ck(cudaMemcpyAsync(c->tcimg.p, c->tc.image.data(), c->tc.image.size(), cudaMemcpyHostToDevice, c->stream), "upload network images");
    ck(cudaStreamSynchronize(c->stream), "upload network images");
    upload_params<float>(c, c->pf);
    upload_params<double>(c, c->pd);
    std::vector<int> po;
    int64_t acc = 0;
    for (auto& s : c->pot.sp) { po.push_back((int)acc); acc += s.nn.size(); }
    upload_ints(c->poff, po, c->stream);
    {
        std::vector<int32_t> map;
        build_param_map(c->plan.pot, c->tc, map);
        std::vector<double> p((size_t)std::max<int64_t>(acc, 1), 0.0);
        c->pot.get_params(p.data());
        c->p64.ensure(8 * p.size());
        c->pmap.ensure(4 * std::max<size_t>(map.size(), 1));
        ck(cudaMemcpyAsync(c->p64.p, p.data(), 8 * p.size(), cudaMemcpyHostToDevice, c->stream), "upload params");
        if (!map.empty()) ck(cudaMemcpyAsync(c->pmap.p, map.data(), 4 * map.size(), cudaMemcpyHostToDevice, c->stream), "upload params");
        ck(cudaStreamSynchronize(c->stream), "upload params");
        c->params_dev_newer = false;
        c->have_grad = false;
    }
    c->have_pot = true;
    c->have_results = false;
    c->have_train = false;
    reset_graph(c);
}

// after optimiser steps on the device the host copy of the parameters is brought up to date
// before anything reads or rebuilds from it
static void sync_params_from_device(ann_ctx* c) {
    if (!c->params_dev_newer) return;
    std::vector<double> p((size_t)c->pot.nparams());
    ck(cudaMemcpyAsync(p.data(), c->p64.p, 8 * p.size(), cudaMemcpyDeviceToHost, c->stream), "D2H params");
    ck(cudaStreamSynchronize(c->stream), "D2H params");
    c->pot.set_params(p.data());
    c->params_dev_newer = false;
}

// ---------------------------------------------------------------- batch buffers
static int estimate_cap(ann_ctx* c, const double* cell) {
    if (c->opt.max_neighbors > 0) return ((c->opt.max_neighbors + 31) / 32) * 32;
    double rho_max = 0.0;
    if (cell) {
        for (int s = 0; s < c->S; ++s) {
            const double* R = cell + 9 * s;
            const double det = R[0] * (R[4] * R[8] - R[7] * R[5]) - R[3] * (R[1] * R[8] - R[7] * R[2]) + R[6] * (R[1] * R[5] - R[4] * R[2]);
            const int n = c->off_h[s + 1] - c->off_h[s];
            if (std::fabs(det) > 0) rho_max = std::max(rho_max, n / std::fabs(det));
        }
    }
    if (rho_max <= 0) rho_max = 0.1;
    const double rc = c->pot.rc + (c->md_ready ? c->md_skin : 0.0);
    const double est = rho_max * 4.18879 * rc * rc * rc;
    int cap = (int)(est * 1.5 + 32);
    return std::min(((cap + 31) / 32) * 32, 4096);
}
static void ensure_batch_buffers(ann_ctx* c) {
    const int S = c->S, N = std::max(c->N, 1), T = c->pot.ntypes(), imax = c->pot.max_input();
    const size_t rb = sizeof(double);  // sized for the widest precision
    c->cell.ensure(sizeof(double) * 9 * std::max(S, 1));
    c->pos.ensure(sizeof(double) * 3 * N); c->type.ensure(sizeof(int32_t) * N); c->sid.ensure(sizeof(int32_t) * N);
    c->geo.ensure(sizeof(StrucGeo) * std::max(S, 1));
    c->nbins_cap = 2 * N + S + 2;
    c->pos4.ensure(sizeof(float4) * N); c->abin.ensure(4 * N); c->abc.ensure(4 * N); c->am.ensure(4 * N); c->aslot.ensure(4 * N);
    c->bcount.ensure(4 * (size_t)(c->nbins_cap + 1)); c->bstart.ensure(4 * (size_t)(c->nbins_cap + 1));
    c->bidx.ensure(4 * N); c->bm.ensure(4 * N); c->bpos4.ensure(sizeof(float4) * N); c->bposd.ensure(sizeof(double) * 3 * N);
    c->nbins_total.ensure(4); c->nn.ensure(4 * N); c->ntc.ensure(4 * (size_t)N * T);
    c->nj.ensure(4 * (size_t)N * c->cap); c->nimg.ensure(4 * (size_t)N * c->cap); c->nr.ensure(sizeof(Vec4d) * (size_t)N * c->cap);
    c->scan_tmp.ensure(4 * scan_tmp_ints(c->nbins_cap + 1)); c->counter.ensure(16); c->status.ensure(4 * 8);
    c->G.ensure(rb * (size_t)N * std::max(imax, 1)); c->dEdG.ensure(rb * (size_t)N * std::max(imax, 1));
    c->Eatom.ensure(sizeof(double) * N); c->F.ensure(rb * 3 * (size_t)N); c->W.ensure(rb * 9 * (size_t)N);
    c->Es.ensure(sizeof(double) * std::max(S, 1)); c->Ws.ensure(sizeof(double) * 9 * std::max(S, 1)); c->Fout.ensure(sizeof(double) * 3 * (size_t)N);
    c->tcount.ensure(4 * ((size_t)T + 1 + N)); c->tstart.ensure(4 * ((size_t)T + 1)); c->tlist.ensure(4 * (size_t)N);
}

static void stage_offsets(ann_ctx* c, int nstruc, const int64_t* atom_offsets) {
    if (nstruc < 0) throw ann_error(ANN_ERR_ARG, "nstruc must be >= 0");
    if (!atom_offsets) throw ann_error(ANN_ERR_ARG, "atom_offsets is NULL");
    if (atom_offsets[0] != 0) throw ann_error(ANN_ERR_ARG, "atom_offsets[0] must be 0");
    for (int s = 0; s < nstruc; ++s)
        if (atom_offsets[s + 1] < atom_offsets[s]) throw ann_error(ANN_ERR_ARG, "atom_offsets must be non-decreasing");
    if (atom_offsets[nstruc] > (int64_t)1 << 30) throw ann_error(ANN_ERR_ARG, "too many atoms in one batch (max 2^30)");
    c->S = nstruc;
    c->N = (int)atom_offsets[nstruc];
    c->off_h.assign(nstruc + 1, 0);
    for (int s = 0; s <= nstruc; ++s) c->off_h[s] = (int32_t)atom_offsets[s];
    // chunks of the per-structure reductions
    c->rchunk_h.clear();
    c->rschunk_h.assign(nstruc + 1, 0);
    for (int s = 0; s < nstruc; ++s) {
        c->rschunk_h[s] = (int32_t)(c->rchunk_h.size() / 3);
        for (int a = c->off_h[s]; a < c->off_h[s + 1]; a += RED_CHUNK) {
            c->rchunk_h.push_back(s); c->rchunk_h.push_back(a); c->rchunk_h.push_back(std::min(a + RED_CHUNK, c->off_h[s + 1]));
        }
    }
    c->rschunk_h[nstruc] = (int32_t)(c->rchunk_h.size() / 3);
}

// a batch staged by the compute or training calls replaces the MD system: the MD state (list skin,
// velocities) no longer applies, and ann_md_init starts a new one
static void leave_md(ann_ctx* c) {
    if (!c->md_ready) return;
    c->md_ready = false;
    c->cap = 0;   // re-estimated without the skin
}

static void upload_batch(ann_ctx* c, int nstruc, const int64_t* offs, const double* posn, const int32_t* type, const double* cell, bool device_src) {
    if (!c->have_pot) throw ann_error(ANN_ERR_STATE, "no potential loaded");
    stage_offsets(c, nstruc, offs);
    if (c->N > 0 && (!posn || !type)) throw ann_error(ANN_ERR_ARG, "posn/type is NULL");
    if (nstruc > 0 && !cell) throw ann_error(ANN_ERR_ARG, "cell is NULL");
    // types and positions are checked on the device (ST_BAD_TYPE, ST_NONFINITE), cells here
    if (!device_src) {
        for (int64_t k = 0; k < 9 * (int64_t)nstruc; ++k) if (!std::isfinite(cell[k])) throw ann_error(ANN_ERR_NUMERIC, "non-finite cell");
        for (int s = 0; s < nstruc; ++s) {
            const double* R = cell + 9 * s;
            const double det = R[0] * (R[4] * R[8] - R[7] * R[5]) - R[3] * (R[1] * R[8] - R[7] * R[2]) + R[6] * (R[1] * R[5] - R[4] * R[2]);
            if (!(std::fabs(det) > 0)) throw ann_error(ANN_ERR_ARG, "singular cell of structure " + std::to_string(s));
        }
    }
    if (c->cap == 0) c->cap = estimate_cap(c, device_src ? nullptr : cell);
    ensure_batch_buffers(c);
    const cudaMemcpyKind k = device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    {
        // offsets, the reduction chunks and the structures' first chunks in one copy (pageable
        // copies return once the host data is staged). The chunk buffers are sized by the bound
        // S + N / RED_CHUNK + 1, so that a captured graph's pointers stay valid for every batch
        // with the same S and N.
        const size_t nmax = (size_t)c->S + (size_t)c->N / RED_CHUNK + 1;
        const size_t o_ch = (size_t)c->S + 1, o_sc = o_ch + 3 * nmax;
        c->tables_h.assign(o_sc + c->S + 1, 0);
        std::copy(c->off_h.begin(), c->off_h.end(), c->tables_h.begin());
        std::copy(c->rchunk_h.begin(), c->rchunk_h.end(), c->tables_h.begin() + o_ch);
        std::copy(c->rschunk_h.begin(), c->rschunk_h.end(), c->tables_h.begin() + o_sc);
        c->tables.ensure(4 * c->tables_h.size());
        c->rpartial.ensure(sizeof(double) * 10 * nmax);
        ck(cudaMemcpyAsync(c->tables.p, c->tables_h.data(), 4 * c->tables_h.size(), cudaMemcpyHostToDevice, c->stream), "H2D offsets");
        c->off_d = c->tables.as<int32_t>();
        c->rchunk_d = c->off_d + o_ch;
        c->rschunk_d = c->off_d + o_sc;
    }
    if (c->N > 0) {
        launch_fill_sid(c->S, c->off_d, c->sid.as<int32_t>(), c->stream);
        ck(cudaMemcpyAsync(c->pos.p, posn, sizeof(double) * 3 * (size_t)c->N, k, c->stream), "copy positions");
        ck(cudaMemcpyAsync(c->type.p, type, sizeof(int32_t) * (size_t)c->N, k, c->stream), "copy types");
    }
    if (c->S > 0) ck(cudaMemcpyAsync(c->cell.p, cell, sizeof(double) * 9 * (size_t)c->S, k, c->stream), "copy cells");
    c->have_batch = true;
    c->have_results = false;
}

// ---------------------------------------------------------------- the E+F kernel sequence
template <typename real>
static BpArgs<real> bp_args(ann_ctx* c) {
    BpArgs<real> b{};
    b.natoms = c->N; b.ntypes = c->pot.ntypes(); b.cap = c->cap; b.newton_untranslated = (c->opt.newton == ANN_NEWTON_UNTRANSLATED);
    b.type = c->type.as<int32_t>(); b.nn = c->nn.as<int32_t>(); b.ntc = c->ntc.as<int32_t>(); b.nj = c->nj.as<int32_t>(); b.nimg = c->nimg.as<int32_t>();
    b.nr = c->nr.p; b.G = c->G.as<real>(); b.dEdG = c->dEdG.as<real>(); b.F = c->F.as<real>(); b.W = c->W.as<real>();
    b.lam = c->lam.as<real>(); b.U = c->U.as<real>();
    b.counter = c->counter.as<uint32_t>(); b.status = c->status.as<int32_t>();
    return b;
}
static NbrArgs nbr_args(ann_ctx* c, double rc) {
    NbrArgs a{};
    a.nstruc = c->S; a.natoms = c->N; a.ntypes = c->pot.ntypes(); a.cap = c->cap; a.rc = rc;
    a.off = c->off_d; a.cell = c->cell.as<double>(); a.pos = c->pos.as<double>(); a.type = c->type.as<int32_t>(); a.sid = c->sid.as<int32_t>();
    a.geo = c->geo.as<StrucGeo>(); a.pos4 = c->pos4.as<float4>(); a.abin = c->abin.as<int32_t>(); a.abc = c->abc.as<int32_t>(); a.am = c->am.as<int32_t>();
    a.aslot = c->aslot.as<int32_t>(); a.bcount = c->bcount.as<int32_t>(); a.bstart = c->bstart.as<int32_t>(); a.bidx = c->bidx.as<int32_t>();
    a.bm = c->bm.as<int32_t>(); a.bpos4 = c->bpos4.as<float4>(); a.bposd = c->bposd.as<double>(); a.nbins_cap = c->nbins_cap;
    a.nbins_total = c->nbins_total.as<int32_t>(); a.nn = c->nn.as<int32_t>(); a.ntc = c->ntc.as<int32_t>(); a.nj = c->nj.as<int32_t>();
    a.nimg = c->nimg.as<int32_t>(); a.nr = c->nr.p; a.scan_tmp = c->scan_tmp.as<int32_t>(); a.counter = c->counter.as<uint32_t>();
    a.status = c->status.as<int32_t>();
    return a;
}

// diagnostics: in debug mode every phase is synchronised and checked, so that a failing
// launch is reported with its phase name
static void check_phase(ann_ctx* c, const char* name) {
    if (!c->debug) return;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) throw ann_error(ANN_ERR_CUDA, std::string("phase '") + name + "': " + cudaGetErrorString(e));
}

static void mark(ann_ctx* c, int k) {
    if (!c->profile) return;
    if (!c->ev[k]) cudaEventCreate(&c->ev[k]);
    cudaEventRecord(c->ev[k], c->stream);
}

static RedTable red_table(ann_ctx* c) {
    RedTable t;
    t.nchunks = (int32_t)(c->rchunk_h.size() / 3);
    t.chunk = c->rchunk_d; t.schunk = c->rschunk_d; t.partial = c->rpartial.as<double>();
    return t;
}

// the MIXED network pass runs on the tensor cores unless the SIMT kernels are asked for
static bool use_tc(const ann_ctx* c) { return c->opt.mlp_backend != 1 && c->tc.ok; }

// the network stage: per-atom energies and dE/dG of natoms atoms grouped by type (tstart/tlist)
template <typename real>
static void enqueue_networks(ann_ctx* c, int natoms, DevBuf& G, DevBuf& dEdG, DevBuf& Eatom, DevBuf& tstart, DevBuf& tlist,
                             const DevParams<real>& prm) {
    const DevPot& pot = c->plan.pot;
    if (!std::is_same<real, double>::value && use_tc(c)) {
        for (int ty = 0; ty < c->pot.ntypes(); ++ty) {
            TcArgs ta{};
            ta.natoms = natoms; ta.imax = pot.imax; ta.type = ty;
            ta.tstart = tstart.as<int32_t>(); ta.tlist = tlist.as<int32_t>();
            ta.G = G.as<float>(); ta.dEdG = dEdG.as<float>(); ta.Eatom = Eatom.as<double>();
            ta.image = c->tcimg.as<uint8_t>(); ta.status = c->status.as<int32_t>();
            launch_mlp_tc(c->tc.t[ty], ta, c->tc.smem_bytes(ty), c->stream);
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

template <typename real>
static void enqueue_ef(ann_ctx* c, bool forces, bool build_list) {
    cudaStream_t st = c->stream;
    const bool fp64 = std::is_same<real, double>::value;
    const DevPot& pot = c->plan.pot;
    // the per-type atom lists depend on the types only: outside the phase-timed and debug modes
    // they run on a side stream that forks here and joins before the networks (a parallel branch
    // of the captured graph, beside the neighbour search and the symmetry functions)
    const bool side = !c->profile && !c->debug;
    auto type_lists = [&](cudaStream_t s) {
        launch_type_lists(c->N, c->pot.ntypes(), c->type.as<int32_t>(), c->tcount.as<int32_t>(), c->tstart.as<int32_t>(),
                          c->tlist.as<int32_t>(), c->status.as<int32_t>(), s);
    };
    if (side) {
        ck(cudaEventRecord(c->ev_fork, st), "event record");
        ck(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "stream wait");
        type_lists(c->side);
        ck(cudaEventRecord(c->ev_join, c->side), "event record");
    }
    mark(c, 0);
    if (build_list) launch_neighbors(nbr_args(c, c->pot.rc + (c->md_ready ? c->md_skin : 0.0)), fp64, st);
    else launch_refresh_geometry(nbr_args(c, c->pot.rc + c->md_skin), fp64, st);
    check_phase(c, "neighbour list");
    mark(c, 1);
    if (!side) type_lists(st);
    check_phase(c, "type lists");
    mark(c, 2);
    BpArgs<real> b = bp_args<real>(c);
    b.prm = params_of<real>(c->pf, c->pd);
    launch_symm<real>(pot, b, st);
    check_phase(c, "symmetry functions");
    mark(c, 3);
    if (side) ck(cudaStreamWaitEvent(st, c->ev_join, 0), "stream wait");
    enqueue_networks<real>(c, c->N, c->G, c->dEdG, c->Eatom, c->tstart, c->tlist, b.prm);
    check_phase(c, "networks");
    mark(c, 4);
    if (forces) {
        cudaMemsetAsync(c->F.p, 0, sizeof(real) * 3 * (size_t)std::max(c->N, 1), st);
        launch_force<real>(pot, b, st);
    }
    check_phase(c, "forces");
    mark(c, 5);
    launch_reduce_structures<real>(c->S, red_table(c), c->Eatom.as<double>(), forces ? c->W.as<real>() : nullptr,
                                   c->F.as<real>(), c->Es.as<double>(), c->Ws.as<double>(), forces ? c->Fout.as<double>() : nullptr, st);
    check_phase(c, "reductions");
    mark(c, 6);
}

static void run_batch(ann_ctx* c, int prec, bool forces, bool build_list = true) {
    if (!c->have_batch) throw ann_error(ANN_ERR_STATE, "no batch staged");
    if (prec != ANN_FP64 && prec != ANN_MIXED) throw ann_error(ANN_ERR_ARG, "invalid precision");
    ck(cudaMemsetAsync(c->status.p, 0, 4 * 8, c->stream), "memset status");
    // shared-memory needs of this batch (neighbour rows are staged per warp)
    const size_t need_bp = bp_smem_bytes(c->plan.pot, c->cap, prec == ANN_FP64) + 1024;
    const size_t need_mlp = mlp_smem_bytes(c->plan.pot, prec == ANN_FP64, false) + 1024;
    if (need_bp > (size_t)c->max_smem)
        throw ann_error(ANN_ERR_CAPACITY, "neighbour capacity " + std::to_string(c->cap) + " needs " + std::to_string(need_bp) +
                                              " B of shared memory per block (device limit " + std::to_string(c->max_smem) + ")");
    if (!(prec == ANN_MIXED && use_tc(c)) && need_mlp > (size_t)c->max_smem)
        throw ann_error(ANN_ERR_UNSUPPORTED, "networks too wide for the shared-memory network kernel");
    const GraphKey key{c->S, c->N, c->cap, prec, forces ? 1 : 0, c->nbins_cap, (int)(c->rchunk_h.size() / 3), g_alloc_gen.load()};
    const bool graphs = c->opt.use_graphs && c->N > 0 && !c->profile;
    const int gs = build_list ? 0 : 1;
    if (graphs) {
        if (!(c->gexec[gs] && c->gkey[gs] == key)) {
            if (c->gexec[gs]) { cudaGraphExecDestroy(c->gexec[gs]); c->gexec[gs] = nullptr; }
            cudaGraph_t g = nullptr;
            const int64_t before = g_launch_counter;
            ck(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            if (prec == ANN_FP64) enqueue_ef<double>(c, forces, build_list); else enqueue_ef<float>(c, forces, build_list);
            const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
            if (ce != cudaSuccess) {
                // locate the failing launch: replay the sequence eagerly with per-phase checks
                cudaGetLastError();
                if (g) cudaGraphDestroy(g);
                const bool d0 = c->debug;
                c->debug = true;
                try {
                    if (prec == ANN_FP64) enqueue_ef<double>(c, forces, build_list); else enqueue_ef<float>(c, forces, build_list);
                } catch (...) { c->debug = d0; throw; }
                c->debug = d0;
                throw ann_error(ANN_ERR_CUDA, std::string("graph capture failed (") + cudaGetErrorString(ce) + ") but the eager replay succeeded");
            }
            c->graph_kernels[gs] = g_launch_counter - before;
            ck(cudaGraphInstantiate(&c->gexec[gs], g, 0), "graph instantiate");
            cudaGraphDestroy(g);
            c->gkey[gs] = key;
        }
        ck(cudaGraphLaunch(c->gexec[gs], c->stream), "graph launch");
        c->kernels += c->graph_kernels[gs];
    } else {
        const int64_t before = g_launch_counter;
        if (prec == ANN_FP64) enqueue_ef<double>(c, forces, build_list); else enqueue_ef<float>(c, forces, build_list);
        c->kernels += g_launch_counter - before;
    }
    ck(cudaGetLastError(), "kernel launch");
    c->last_prec = prec;
    c->have_results = true;
    c->have_forces = forces;
}

// a page-locked copy of the device status word, for reads that ride along with result copies
static int32_t* status_host(ann_ctx* c) {
    if (!c->status_h) ck(cudaMallocHost(reinterpret_cast<void**>(&c->status_h), 4 * 8), "cudaMallocHost status");
    return c->status_h;
}

// wait for the batch; on neighbour overflow grow the capacity and recompute
static void finish_batch(ann_ctx* c) {
    for (int attempt = 0; attempt < 6; ++attempt) {
        int32_t st[8];
        ck(cudaMemcpyAsync(st, c->status.p, sizeof(st), cudaMemcpyDeviceToHost, c->stream), "D2H status");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        if (st[0] == 0) return;
        if (st[0] & ST_BAD_TYPE) throw ann_error(ANN_ERR_ARG, "type index out of range");
        if (st[0] & ST_NONFINITE) throw ann_error(ANN_ERR_NUMERIC, "non-finite position or singular cell");
        if (st[0] & ST_IMAGE_RANGE) throw ann_error(ANN_ERR_ARG, "an atom lies more than 500 cell lengths outside its cell");
        if (st[0] & ST_TIMEOUT) throw ann_error(ANN_ERR_TIMEOUT, "a bounded device wait gave up");
        if (st[0] & ST_NBR_OVERFLOW) {
            const int need = std::max(st[1], c->cap + 1);
            const int ncap = ((int)(need * 1.25) + 31) / 32 * 32;
            if (ncap > 8192) throw ann_error(ANN_ERR_CAPACITY, "more than 8192 neighbours per atom");
            c->cap = ncap;
            ensure_batch_buffers(c);
            reset_graph(c);
            run_batch(c, c->last_prec, c->have_forces);
            continue;
        }
        throw ann_error(ANN_ERR_CUDA, "unknown device status " + std::to_string(st[0]));
    }
    throw ann_error(ANN_ERR_CAPACITY, "neighbour capacity could not be grown");
}

// ---------------------------------------------------------------- extern "C"
extern "C" {

void ann_default_options(ann_options* o) {
    if (!o) return;
    o->device = 0; o->precision = ANN_MIXED; o->newton = ANN_NEWTON_ALL_IMAGES; o->max_neighbors = 0; o->use_graphs = 1; o->mlp_backend = 0;
}
int ann_abi_version(void) { return ANN_GPU_ABI_VERSION; }

int ann_create(ann_ctx** out, const ann_options* opt) {
    if (!out) return fail(nullptr, ANN_ERR_ARG, "ctx pointer is NULL");
    *out = nullptr;
    ann_ctx* c = new ann_ctx();
    ann_default_options(&c->opt);
    if (opt) c->opt = *opt;
    try {
        int n = 0;
        ck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (c->opt.device < 0 || c->opt.device >= n) throw ann_error(ANN_ERR_CUDA, "CUDA device " + std::to_string(c->opt.device) + " not available");
        set_device(c);
        ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream create");
        ck(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking), "stream create");
        ck(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "event create");
        ck(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "event create");
        configure_kernels();
        cudaDeviceGetAttribute(&c->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->opt.device);
        cudaDeviceGetAttribute(&c->tc.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->opt.device);
        if (c->opt.mlp_backend < 0 || c->opt.mlp_backend > 2) throw ann_error(ANN_ERR_ARG, "mlp_backend must be 0, 1 or 2");
        const char* dbg = std::getenv("ANN_DEBUG");
        c->debug = dbg && dbg[0] == '1';
        if (c->debug) c->opt.use_graphs = 0;
    } catch (ann_error& e) {
        if (c->stream) cudaStreamDestroy(c->stream);
        if (c->side) cudaStreamDestroy(c->side);
        if (c->ev_fork) cudaEventDestroy(c->ev_fork);
        if (c->ev_join) cudaEventDestroy(c->ev_join);
        delete c;
        return fail(nullptr, e.code, e.what());
    }
    *out = c;
    return ANN_OK;
}

int ann_destroy(ann_ctx* c) {
    if (!c) return ANN_OK;
    cudaSetDevice(c->opt.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    reset_graph(c);
    c->pf.release(); c->pd.release();
    for (DevBuf* b : {&c->poff, &c->cell, &c->pos, &c->type, &c->sid, &c->geo, &c->pos4, &c->abin, &c->abc, &c->am, &c->aslot,
                      &c->bcount, &c->bstart, &c->bidx, &c->bm, &c->bpos4, &c->bposd, &c->nbins_total, &c->nn, &c->ntc, &c->nj, &c->nimg,
                      &c->nr, &c->scan_tmp, &c->counter, &c->status, &c->G, &c->dEdG, &c->Eatom, &c->F, &c->W, &c->Es, &c->Ws, &c->Fout,
                      &c->tcount, &c->tstart, &c->tlist, &c->Eref, &c->Fref, &c->loss3, &c->ce, &c->lam, &c->U, &c->grad,
                      &c->vel, &c->minv, &c->mass, &c->disp_ref, &c->mdflag, &c->ke, &c->md_R_d, &c->md_Ri_d,
                      &c->tables, &c->rpartial, &c->tcimg, &c->p64, &c->pmap, &c->adam_m, &c->adam_v,
                      &c->lx, &c->ltype, &c->lilist, &c->lnoff, &c->lneigh, &c->lrtype, &c->lnn, &c->lntc, &c->lnj, &c->lnr, &c->lG,
                      &c->ldEdG, &c->lEatom, &c->lF, &c->lW, &c->lFout, &c->ltcount, &c->ltstart, &c->ltlist, &c->ltables, &c->lpartial,
                      &c->lEs, &c->lWs, &c->st_acc, &c->st_n, &c->st_part, &c->st_pcount})
        b->release();
    for (auto& e : c->ev) if (e) cudaEventDestroy(e);
    if (c->status_h) cudaFreeHost(c->status_h);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    delete c;
    return ANN_OK;
}

const char* ann_last_error(const ann_ctx* c) {
    if (c) return c->err.c_str();
    std::lock_guard<std::mutex> g(g_err_mu);
    return g_err.c_str();
}

int ann_load_potential_text(ann_ctx* c, const char* text) {
    if (!c || !text) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        Potential p;
        p.read_text(text);
        p.validate();
        c->pot = p;
        c->adam_ready = false;
        c->st_ready = false;   // statistics belong to the previous potential's inputs
        rebuild_plan(c);
    })
}
int ann_load_potential(ann_ctx* c, const char* path) {
    if (!c || !path) return fail(c, ANN_ERR_ARG, "NULL argument");
    std::ifstream f(path);
    if (!f) return fail(c, ANN_ERR_IO, std::string("could not open potential file: \"") + path + "\"");
    std::stringstream ss;
    ss << f.rdbuf();
    return ann_load_potential_text(c, ss.str().c_str());
}
int ann_write_potential(ann_ctx* c, const char* path) {
    if (!c || !path) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    std::ofstream f(path);
    if (!f) return fail(c, ANN_ERR_IO, std::string("could not write potential file: \"") + path + "\"");
    try { set_device(c); sync_params_from_device(c); } catch (ann_error& e) { return fail(c, e.code, e.what()); }
    f << c->pot.write_text();
    return f.good() ? ANN_OK : fail(c, ANN_ERR_IO, "write failed");
}
int ann_num_types(ann_ctx* c, int32_t* n) {
    if (!c || !n) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    *n = c->pot.ntypes();
    return ANN_OK;
}
int ann_type_index(ann_ctx* c, const char* name, int32_t* idx) {
    if (!c || !name || !idx) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    auto it = c->pot.index.find(name);
    if (it == c->pot.index.end()) return fail(c, ANN_ERR_ARG, std::string("unknown type name: ") + name);
    *idx = it->second;
    return ANN_OK;
}
int ann_type_name(ann_ctx* c, int32_t i, char* buf, int32_t len) {
    if (!c || !buf || len <= 0) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (i < 0 || i >= c->pot.ntypes()) return fail(c, ANN_ERR_ARG, "type index out of range");
    std::snprintf(buf, len, "%s", c->pot.sp[i].name.c_str());
    return ANN_OK;
}
int ann_cutoff(ann_ctx* c, double* rc) {
    if (!c || !rc) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    *rc = c->pot.rc;
    return ANN_OK;
}
int ann_num_inputs(ann_ctx* c, int32_t t, int32_t* n) {
    if (!c || !n) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (t < 0 || t >= c->pot.ntypes()) return fail(c, ANN_ERR_ARG, "type index out of range");
    *n = c->pot.sp[t].nInput;
    return ANN_OK;
}
int ann_num_params(ann_ctx* c, int64_t* n) {
    if (!c || !n) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    *n = c->pot.nparams();
    return ANN_OK;
}
int ann_get_params(ann_ctx* c, double* p, int64_t n) {
    if (!c || !p) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (n != c->pot.nparams()) return fail(c, ANN_ERR_ARG, "parameter count mismatch");
    ANN_TRY(c, { set_device(c); sync_params_from_device(c); c->pot.get_params(p); })
}
int ann_set_params(ann_ctx* c, const double* p, int64_t n) {
    if (!c || !p) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (n != c->pot.nparams()) return fail(c, ANN_ERR_ARG, "Invalid size: vector and network mismatch.");  // nn.cpp:869
    ANN_TRY(c, { set_device(c); c->pot.set_params(p); rebuild_plan(c); })
}
int ann_set_input_scaling(ann_ctx* c, int32_t t, const double* w, const double* b, int32_t n) {
    if (!c || !w || !b) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (t < 0 || t >= c->pot.ntypes()) return fail(c, ANN_ERR_ARG, "type index out of range");
    if (n != c->pot.sp[t].nInput) return fail(c, ANN_ERR_ARG, "input count mismatch");
    ANN_TRY(c, {
        set_device(c);
        sync_params_from_device(c);
        c->pot.sp[t].nn.inpw.assign(w, w + n);
        c->pot.sp[t].nn.inpb.assign(b, b + n);
        rebuild_plan(c);
    })
}
int ann_init_network(ann_ctx* c, int32_t t, int32_t seed, int32_t dist, int32_t init, double sb, double sw) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (t < 0 || t >= c->pot.ntypes()) return fail(c, ANN_ERR_ARG, "type index out of range");
    ANN_TRY(c, { set_device(c); sync_params_from_device(c); init_network(c->pot.sp[t].nn, seed, dist, init, sb, sw); rebuild_plan(c); })
}

int ann_batch_upload(ann_ctx* c, int32_t nstruc, const int64_t* offs, const double* posn, const int32_t* type, const double* cell) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, { set_device(c); leave_md(c); upload_batch(c, nstruc, offs, posn, type, cell, false); })
}
int ann_batch_set_device(ann_ctx* c, int32_t nstruc, const int64_t* offs, const double* d_posn, const int32_t* d_type, const double* d_cell) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, { set_device(c); leave_md(c); upload_batch(c, nstruc, offs, d_posn, d_type, d_cell, true); })
}
int ann_batch_compute(ann_ctx* c, int32_t prec, int32_t want_forces) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, { set_device(c); run_batch(c, prec, want_forces != 0); })
}
int ann_batch_download(ann_ctx* c, double* energy, double* forces, double* virial) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        finish_batch(c);
        if ((forces || virial) && !c->have_forces) throw ann_error(ANN_ERR_STATE, "forces were not computed for this batch");
        if (energy && c->S > 0) ck(cudaMemcpyAsync(energy, c->Es.p, sizeof(double) * c->S, cudaMemcpyDeviceToHost, c->stream), "D2H energy");
        if (forces && c->N > 0) ck(cudaMemcpyAsync(forces, c->Fout.p, sizeof(double) * 3 * (size_t)c->N, cudaMemcpyDeviceToHost, c->stream), "D2H forces");
        if (virial && c->S > 0) ck(cudaMemcpyAsync(virial, c->Ws.p, sizeof(double) * 9 * (size_t)c->S, cudaMemcpyDeviceToHost, c->stream), "D2H virial");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
    })
}
int ann_batch_results_device(ann_ctx* c, double* e, double* f, double* w) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        finish_batch(c);
        if (e && c->S > 0) ck(cudaMemcpyAsync(e, c->Es.p, sizeof(double) * c->S, cudaMemcpyDeviceToDevice, c->stream), "D2D energy");
        if (f && c->N > 0) ck(cudaMemcpyAsync(f, c->Fout.p, sizeof(double) * 3 * (size_t)c->N, cudaMemcpyDeviceToDevice, c->stream), "D2D forces");
        if (w && c->S > 0) ck(cudaMemcpyAsync(w, c->Ws.p, sizeof(double) * 9 * (size_t)c->S, cudaMemcpyDeviceToDevice, c->stream), "D2D virial");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
    })
}
int ann_kernel_count(ann_ctx* c, int64_t* n) {
    if (!c || !n) return fail(c, ANN_ERR_ARG, "NULL argument");
    *n = c->kernels;
    return ANN_OK;
}
int ann_profile_phases(ann_ctx* c, int32_t enable) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    c->profile = enable != 0;
    return ANN_OK;
}
int ann_phase_times(ann_ctx* c, double* ms, int32_t n) {
    if (!c || !ms) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (!c->profile || !c->ev[6]) throw ann_error(ANN_ERR_STATE, "enable ann_profile_phases and run a batch first");
        ck(cudaEventSynchronize(c->ev[6]), "event sync");
        for (int k = 0; k < n && k < 6; ++k) {
            float t = 0.f;
            ck(cudaEventElapsedTime(&t, c->ev[k], c->ev[k + 1]), "event elapsed");
            ms[k] = t;
        }
    })
}
int ann_synchronize(ann_ctx* c) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, { set_device(c); ck(cudaStreamSynchronize(c->stream), "synchronize"); })
}
void* ann_stream(ann_ctx* c) { return c ? (void*)c->stream : nullptr; }

int ann_compute(ann_ctx* c, int32_t nstruc, const int64_t* offs, const double* posn, const int32_t* type, const double* cell,
                double* energy, double* forces, double* virial, int32_t prec) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (!energy) return fail(c, ANN_ERR_ARG, "energy is NULL");
    ANN_TRY(c, {
        set_device(c);
        leave_md(c);
        upload_batch(c, nstruc, offs, posn, type, cell, false);
        run_batch(c, prec, forces != nullptr || virial != nullptr);
        // the results and the status word in one round trip; a status that is not clean (list
        // overflow, bad input) goes through finish_batch, which recovers or throws, and the
        // results are copied again
        auto copy_out = [&]() {
            if (c->S > 0) ck(cudaMemcpyAsync(energy, c->Es.p, sizeof(double) * c->S, cudaMemcpyDeviceToHost, c->stream), "D2H energy");
            if (forces && c->N > 0) ck(cudaMemcpyAsync(forces, c->Fout.p, sizeof(double) * 3 * (size_t)c->N, cudaMemcpyDeviceToHost, c->stream), "D2H forces");
            if (virial && c->S > 0) ck(cudaMemcpyAsync(virial, c->Ws.p, sizeof(double) * 9 * (size_t)c->S, cudaMemcpyDeviceToHost, c->stream), "D2H virial");
        };
        copy_out();
        int32_t* sh = status_host(c);
        ck(cudaMemcpyAsync(sh, c->status.p, 4 * 8, cudaMemcpyDeviceToHost, c->stream), "D2H status");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        if (sh[0] != 0) {
            finish_batch(c);
            copy_out();
            ck(cudaStreamSynchronize(c->stream), "synchronize");
        }
    })
}

}  // extern "C"

// ---- a caller's neighbour list: LAMMPS pair style shape (full list over local + ghost atoms)
// The sequence of one list call: type lists, symmetry functions, networks, forces, the energy and
// virial sums over the rows, and the FP64 copy of the forces of all nall atoms. It runs eagerly:
// an MD engine's list and ghost count change at every reneighbouring.
template <typename real>
static void enqueue_list(ann_ctx* c, int nrows, int nall, int cap, int nchunks, bool forces, bool have_ilist) {
    cudaStream_t st = c->stream;
    const DevPot& pot = c->plan.pot;
    const int T = c->pot.ntypes();
    launch_type_lists(nrows, T, c->lrtype.as<int32_t>(), c->ltcount.as<int32_t>(), c->ltstart.as<int32_t>(), c->ltlist.as<int32_t>(),
                      c->status.as<int32_t>(), st);
    BpArgs<real> b{};
    b.natoms = nrows; b.ntypes = T; b.cap = cap; b.newton_untranslated = 0;
    b.type = c->lrtype.as<int32_t>(); b.nn = c->lnn.as<int32_t>(); b.ntc = c->lntc.as<int32_t>(); b.nj = c->lnj.as<int32_t>();
    b.nimg = nullptr; b.nr = c->lnr.p;
    b.G = c->lG.as<real>(); b.dEdG = c->ldEdG.as<real>(); b.F = c->lF.as<real>(); b.W = c->lW.as<real>();
    b.self = have_ilist ? c->lilist.as<int32_t>() : nullptr;
    b.counter = c->counter.as<uint32_t>(); b.status = c->status.as<int32_t>();
    b.prm = params_of<real>(c->pf, c->pd);
    launch_symm<real>(pot, b, st);
    enqueue_networks<real>(c, nrows, c->lG, c->ldEdG, c->lEatom, c->ltstart, c->ltlist, b.prm);
    if (forces) {
        cudaMemsetAsync(c->lF.p, 0, sizeof(real) * 3 * (size_t)std::max(nall, 1), st);
        launch_force<real>(pot, b, st);
    }
    RedTable t;
    t.nchunks = nchunks; t.schunk = c->ltables.as<int32_t>(); t.chunk = t.schunk + 2; t.partial = c->lpartial.as<double>();
    launch_reduce_structures<real>(1, t, c->lEatom.as<double>(), forces ? c->lW.as<real>() : nullptr, c->lF.as<real>(),
                                   c->lEs.as<double>(), c->lWs.as<double>(), nullptr, st);
    if (forces) launch_to_double<real>(3 * (size_t)nall, c->lF.as<real>(), c->lFout.as<double>(), st);
}

extern "C" {
int ann_compute_list(ann_ctx* c, int32_t inum, const int32_t* ilist, const int32_t* numneigh, const int32_t* neigh, int32_t nall,
                     const double* x, const int32_t* type, double* energy, double* eatom, double* forces, double* virial, int32_t prec,
                     int32_t flags) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (!energy) return fail(c, ANN_ERR_ARG, "energy is NULL");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_pot) throw ann_error(ANN_ERR_STATE, "no potential loaded");
        if (prec != ANN_FP64 && prec != ANN_MIXED) throw ann_error(ANN_ERR_ARG, "invalid precision");
        if (flags & ~ANN_LIST_KEEP) throw ann_error(ANN_ERR_ARG, "unknown flags");
        if (inum < 0 || nall < 0) throw ann_error(ANN_ERR_ARG, "inum and nall must be >= 0");
        const bool keep = (flags & ANN_LIST_KEEP) != 0;
        if (inum > 0 && (!x || nall == 0)) throw ann_error(ANN_ERR_ARG, "x is NULL, or nall is 0");
        cudaStream_t st = c->stream;
        if (keep) {
            // the list, ilist and types of the previous call stay on the device: only x is new
            if (!c->list_staged) throw ann_error(ANN_ERR_STATE, "ANN_LIST_KEEP without a list staged by a previous call");
            if (inum != c->list_inum || nall != c->list_nall)
                throw ann_error(ANN_ERR_ARG, "ANN_LIST_KEEP: inum / nall differ from the staged list's");
        } else {
            c->list_staged = false;
            if (inum > 0 && (!numneigh || !type)) throw ann_error(ANN_ERR_ARG, "numneigh or type is NULL");
            if (!ilist && inum > nall) throw ann_error(ANN_ERR_ARG, "inum > nall without ilist");
            std::vector<int64_t> noff((size_t)inum + 1, 0);
            int maxnn = 0;
            for (int r = 0; r < inum; ++r) {
                if (numneigh[r] < 0) throw ann_error(ANN_ERR_ARG, "numneigh[" + std::to_string(r) + "] < 0");
                noff[r + 1] = noff[r] + numneigh[r];
                maxnn = std::max(maxnn, numneigh[r]);
            }
            const int64_t M = noff[inum];
            if (M > 0 && !neigh) throw ann_error(ANN_ERR_ARG, "neigh is NULL");
            c->ltype.ensure(4 * (size_t)std::max(nall, 1));
            c->lnoff.ensure(8 * ((size_t)inum + 1)); c->lneigh.ensure(4 * (size_t)std::max<int64_t>(M, 1));
            if (ilist) c->lilist.ensure(4 * (size_t)std::max(inum, 1));
            if (nall > 0) ck(cudaMemcpyAsync(c->ltype.p, type, 4 * (size_t)nall, cudaMemcpyHostToDevice, st), "H2D type");
            ck(cudaMemcpyAsync(c->lnoff.p, noff.data(), 8 * noff.size(), cudaMemcpyHostToDevice, st), "H2D list offsets");
            if (M > 0) ck(cudaMemcpyAsync(c->lneigh.p, neigh, 4 * (size_t)M, cudaMemcpyHostToDevice, st), "H2D neighbours");
            if (ilist && inum > 0) ck(cudaMemcpyAsync(c->lilist.p, ilist, 4 * (size_t)inum, cudaMemcpyHostToDevice, st), "H2D ilist");
            c->list_inum = inum; c->list_nall = nall; c->list_maxnn = maxnn; c->list_have_ilist = ilist != nullptr;
        }
        const bool have_ilist = c->list_have_ilist;
        const int maxnn = c->list_maxnn;
        const bool fp64 = prec == ANN_FP64, want_f = forces != nullptr || virial != nullptr;
        const DevPot& pot = c->plan.pot;
        const int T = c->pot.ntypes(), imax = c->pot.max_input();
        const size_t rb = fp64 ? sizeof(double) : sizeof(float);
        const int64_t launches0 = g_launch_counter;
        c->lx.ensure(sizeof(double) * 3 * (size_t)std::max(nall, 1));
        if (nall > 0) ck(cudaMemcpyAsync(c->lx.p, x, sizeof(double) * 3 * (size_t)nall, cudaMemcpyHostToDevice, st), "H2D x");
        // reduction chunks of the rows: {0, nchunks} then (structure 0, first row, end row) per chunk
        const int nch = (inum + RED_CHUNK - 1) / RED_CHUNK;
        std::vector<int32_t> tab{0, nch};
        for (int r0 = 0; r0 < inum; r0 += RED_CHUNK) { tab.push_back(0); tab.push_back(r0); tab.push_back(std::min(r0 + RED_CHUNK, inum)); }
        c->ltables.ensure(4 * tab.size());
        ck(cudaMemcpyAsync(c->ltables.p, tab.data(), 4 * tab.size(), cudaMemcpyHostToDevice, st), "H2D chunks");
        c->lpartial.ensure(sizeof(double) * 10 * (size_t)std::max(nch, 1)); c->lEs.ensure(8); c->lWs.ensure(72);
        // row capacity: the longest row within rc seen so far plus an eighth, never above the longest
        // given row, and within the shared memory of the symmetry-function / force kernels
        const size_t need_mlp = mlp_smem_bytes(pot, fp64, false) + 1024;
        if (!(prec == ANN_MIXED && use_tc(c)) && need_mlp > (size_t)c->max_smem)
            throw ann_error(ANN_ERR_UNSUPPORTED, "networks too wide for the shared-memory network kernel");
        auto round32 = [](int v) { return ((std::max(v, 1) + 31) / 32) * 32; };
        int capmax = 0;
        while (capmax + 32 <= 8192 && bp_smem_bytes(pot, capmax + 32, fp64) + 1024 <= (size_t)c->max_smem) capmax += 32;
        if (capmax == 0) throw ann_error(ANN_ERR_CAPACITY, "the potential leaves no shared memory for neighbour rows");
        int cap = c->list_hint > 0 ? round32(c->list_hint + c->list_hint / 8 + 1) : round32(maxnn);
        cap = std::min({cap, round32(maxnn), capmax});
        bool done = false;
        for (int attempt = 0; attempt < 4 && !done; ++attempt) {
            c->lrtype.ensure(4 * (size_t)std::max(inum, 1)); c->lnn.ensure(4 * (size_t)std::max(inum, 1));
            c->lntc.ensure(4 * (size_t)std::max(inum, 1) * T); c->lnj.ensure(4 * (size_t)std::max(inum, 1) * cap);
            c->lnr.ensure((fp64 ? sizeof(Vec4d) : sizeof(Vec4f)) * (size_t)std::max(inum, 1) * cap);
            c->lG.ensure(rb * (size_t)std::max(inum, 1) * std::max(imax, 1)); c->ldEdG.ensure(rb * (size_t)std::max(inum, 1) * std::max(imax, 1));
            c->lEatom.ensure(sizeof(double) * std::max(inum, 1)); c->lW.ensure(rb * 9 * (size_t)std::max(inum, 1));
            c->lF.ensure(rb * 3 * (size_t)std::max(nall, 1)); c->lFout.ensure(sizeof(double) * 3 * (size_t)std::max(nall, 1));
            c->ltcount.ensure(4 * ((size_t)T + 1 + std::max(inum, 1))); c->ltstart.ensure(4 * ((size_t)T + 1));
            c->ltlist.ensure(4 * (size_t)std::max(inum, 1));
            c->counter.ensure(16); c->status.ensure(4 * 8);
            ck(cudaMemsetAsync(c->status.p, 0, 4 * 8, st), "memset status");
            ListArgs la{};
            la.nrows = inum; la.nall = nall; la.ntypes = T; la.cap = cap; la.rc2 = c->pot.rc * c->pot.rc; la.hint = c->list_hint;
            la.ilist = have_ilist ? c->lilist.as<int32_t>() : nullptr; la.noff = c->lnoff.as<int64_t>(); la.neigh = c->lneigh.as<int32_t>();
            la.x = c->lx.as<double>(); la.type = c->ltype.as<int32_t>(); la.rtype = c->lrtype.as<int32_t>(); la.nn = c->lnn.as<int32_t>();
            la.ntc = c->lntc.as<int32_t>(); la.nj = c->lnj.as<int32_t>(); la.nr = c->lnr.p; la.status = c->status.as<int32_t>();
            launch_list_rows(la, fp64, st);
            if (fp64) enqueue_list<double>(c, inum, nall, cap, nch, want_f, have_ilist);
            else enqueue_list<float>(c, inum, nall, cap, nch, want_f, have_ilist);
            ck(cudaGetLastError(), "kernel launch");
            int32_t sw[8];
            ck(cudaMemcpyAsync(sw, c->status.p, sizeof(sw), cudaMemcpyDeviceToHost, st), "D2H status");
            ck(cudaStreamSynchronize(st), "synchronize");
            if (sw[2] > c->list_hint) c->list_hint = sw[2];
            if (sw[0] == 0) { done = true; break; }
            if (sw[0] & ST_BAD_INDEX) throw ann_error(ANN_ERR_ARG, "a list or neighbour index is outside [0, nall)");
            if (sw[0] & ST_BAD_TYPE) throw ann_error(ANN_ERR_ARG, "type index out of range");
            if (sw[0] & ST_NONFINITE) throw ann_error(ANN_ERR_NUMERIC, "non-finite position");
            if (sw[0] & ST_TIMEOUT) throw ann_error(ANN_ERR_TIMEOUT, "a bounded device wait gave up");
            if (sw[0] & ST_NBR_OVERFLOW) {
                const int need = std::max(sw[1], cap + 1);
                if (need > capmax)
                    throw ann_error(ANN_ERR_CAPACITY, std::to_string(need) + " neighbours within the cutoff; the shared memory holds " +
                                                          std::to_string(capmax));
                cap = std::min(capmax, round32(need + need / 8));
                continue;
            }
            throw ann_error(ANN_ERR_CUDA, "unknown device status " + std::to_string(sw[0]));
        }
        if (!done) throw ann_error(ANN_ERR_CAPACITY, "neighbour capacity could not be grown");
        c->list_staged = true;
        c->kernels += g_launch_counter - launches0;
        ck(cudaMemcpyAsync(energy, c->lEs.p, sizeof(double), cudaMemcpyDeviceToHost, st), "D2H energy");
        if (eatom && inum > 0) ck(cudaMemcpyAsync(eatom, c->lEatom.p, sizeof(double) * inum, cudaMemcpyDeviceToHost, st), "D2H eatom");
        if (forces && nall > 0) ck(cudaMemcpyAsync(forces, c->lFout.p, sizeof(double) * 3 * (size_t)nall, cudaMemcpyDeviceToHost, st), "D2H forces");
        if (virial) ck(cudaMemcpyAsync(virial, c->lWs.p, sizeof(double) * 9, cudaMemcpyDeviceToHost, st), "D2H virial");
        ck(cudaStreamSynchronize(st), "synchronize");
    })
}

// ---- input statistics and pre-conditioning of a training set (nnptefr2.cpp:686-858)
static void stats_reset(ann_ctx* c) {
    const int T = c->pot.ntypes(), imax = std::max(c->pot.max_input(), 1);
    std::vector<double> a((size_t)T * 6 * imax, 0.0);
    for (int t = 0; t < T; ++t)
        for (int k = 0; k < imax; ++k) { a[((size_t)t * 6) * imax + k] = -DBL_MAX; a[((size_t)t * 6 + 1) * imax + k] = DBL_MAX; }
    c->st_acc.ensure(8 * a.size()); c->st_n.ensure(8 * (size_t)std::max(T, 1));
    ck(cudaMemcpyAsync(c->st_acc.p, a.data(), 8 * a.size(), cudaMemcpyHostToDevice, c->stream), "H2D statistics");
    ck(cudaMemsetAsync(c->st_n.p, 0, 8 * (size_t)std::max(T, 1), c->stream), "memset statistics");
    ck(cudaStreamSynchronize(c->stream), "synchronize");
    c->st_ready = true; c->st_T = T; c->st_imax = imax;
}
// host form of one type's statistics: rows max, min, har, avg, dev, rms of its n inputs
static std::vector<double> stats_host(ann_ctx* c, int t, int64_t* count) {
    const int imax = c->st_imax, n = c->pot.sp[t].nInput;
    std::vector<double> a((size_t)6 * imax), out((size_t)6 * n);
    double N = 0.0;
    ck(cudaMemcpyAsync(a.data(), c->st_acc.as<double>() + (size_t)t * 6 * imax, 8 * a.size(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    ck(cudaMemcpyAsync(&N, c->st_n.as<double>() + t, 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
    ck(cudaStreamSynchronize(c->stream), "synchronize");
    for (int k = 0; k < n; ++k) {
        out[k] = a[k];
        out[n + k] = a[imax + k];
        out[2 * n + k] = N / a[2 * imax + k];
        out[3 * n + k] = a[3 * imax + k] / N;
        out[4 * n + k] = N > 1.0 ? std::sqrt(a[4 * imax + k] / (N - 1.0)) : 0.0;
        out[5 * n + k] = std::sqrt(a[5 * imax + k] / N);
    }
    if (count) *count = (int64_t)N;
    return out;
}

int ann_stats_reset(ann_ctx* c) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    ANN_TRY(c, { set_device(c); stats_reset(c); })
}
int ann_stats_accumulate(ann_ctx* c) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        finish_batch(c);   // a batch still in flight (ann_batch_compute) completes, list overflows recomputed
        if (!c->st_ready || c->st_T != c->pot.ntypes() || c->st_imax != std::max(c->pot.max_input(), 1)) stats_reset(c);
        const int T = c->pot.ntypes(), imax = c->pot.max_input(), maxch = stats_chunks_per_type(c->N);
        if (c->N > 0 && imax > 0) {
            c->st_part.ensure(8 * (size_t)T * maxch * 6 * imax); c->st_pcount.ensure(4 * (size_t)T * maxch);
            const int64_t before = g_launch_counter;
            if (c->last_prec == ANN_FP64)
                launch_input_stats<double>(c->N, T, imax, c->G.as<double>(), c->tstart.as<int32_t>(), c->tlist.as<int32_t>(),
                                           c->st_part.as<double>(), c->st_pcount.as<int32_t>(), c->st_acc.as<double>(), c->st_n.as<double>(), c->stream);
            else
                launch_input_stats<float>(c->N, T, imax, c->G.as<float>(), c->tstart.as<int32_t>(), c->tlist.as<int32_t>(),
                                          c->st_part.as<double>(), c->st_pcount.as<int32_t>(), c->st_acc.as<double>(), c->st_n.as<double>(), c->stream);
            c->kernels += g_launch_counter - before;
            ck(cudaGetLastError(), "statistics kernels");
        }
        ck(cudaStreamSynchronize(c->stream), "synchronize");
    })
}
int ann_stats_get(ann_ctx* c, int32_t t, int64_t* count, double* stats) {
    if (!c || !stats) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (t < 0 || t >= c->pot.ntypes()) return fail(c, ANN_ERR_ARG, "type index out of range");
    ANN_TRY(c, {
        set_device(c);
        if (!c->st_ready || c->st_T != c->pot.ntypes()) throw ann_error(ANN_ERR_STATE, "no statistics accumulated");
        const std::vector<double> h = stats_host(c, t, count);
        std::copy(h.begin(), h.end(), stats);
    })
}
int ann_precondition(ann_ctx* c, int32_t prebias, int32_t prescale, double inbias, double inscale) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (prebias < ANN_PREBIAS_IDENTITY || prebias > ANN_PREBIAS_MIN) return fail(c, ANN_ERR_ARG, "Invalid input bias.");
    if (prescale < ANN_PRESCALE_IDENTITY || prescale > ANN_PRESCALE_MAX) return fail(c, ANN_ERR_ARG, "Invalid input scaling.");
    ANN_TRY(c, {
        set_device(c);
        if (!c->st_ready || c->st_T != c->pot.ntypes()) throw ann_error(ANN_ERR_STATE, "no statistics accumulated");
        sync_params_from_device(c);
        for (int t = 0; t < c->pot.ntypes(); ++t) {
            int64_t N = 0;
            const std::vector<double> h = stats_host(c, t, &N);
            if (N == 0) continue;   // a type without atoms keeps its scaling
            const int n = c->pot.sp[t].nInput;
            const double *mx = h.data(), *mn = mx + n, *har = mx + 2 * n, *avg = mx + 3 * n, *dev = mx + 4 * n, *rms = mx + 5 * n;
            auto& nn = c->pot.sp[t].nn;
            for (int k = 0; k < n; ++k) {
                double b = 0.0, w = 1.0;
                switch (prebias) {
                    case ANN_PREBIAS_MEAN: b = -1.0 * avg[k]; break;
                    case ANN_PREBIAS_HAR: b = -1.0 * har[k]; break;
                    case ANN_PREBIAS_RMS: b = -1.0 * rms[k]; break;
                    case ANN_PREBIAS_MID: b = -0.5 * (mx[k] + mn[k]); break;
                    case ANN_PREBIAS_MIN: b = -1.0 * mn[k]; break;
                    default: b = 0.0; break;
                }
                switch (prescale) {
                    case ANN_PRESCALE_DEV: w = (dev[k] == 0) ? 1.0 : 1.0 / dev[k]; break;
                    case ANN_PRESCALE_MINMAX: { const double s = mx[k] - mn[k]; w = (s > 0) ? 1.0 / s : 1.0; } break;
                    case ANN_PRESCALE_MAX: w = (mx[k] > 0) ? 1.0 / mx[k] : 1.0; break;
                    default: w = 1.0; break;
                }
                nn.inpb[k] = b + inbias;
                nn.inpw[k] = w * inscale;
            }
            nn.outb.assign(nn.outb.size(), 0.0);
            nn.outw.assign(nn.outw.size(), 1.0);
        }
        rebuild_plan(c);
    })
}
int ann_get_input_scaling(ann_ctx* c, int32_t t, double* w, double* b, int32_t n) {
    if (!c || !w || !b) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (t < 0 || t >= c->pot.ntypes()) return fail(c, ANN_ERR_ARG, "type index out of range");
    if (n != c->pot.sp[t].nInput) return fail(c, ANN_ERR_ARG, "input count mismatch");
    std::copy(c->pot.sp[t].nn.inpw.begin(), c->pot.sp[t].nn.inpw.end(), w);
    std::copy(c->pot.sp[t].nn.inpb.begin(), c->pot.sp[t].nn.inpb.end(), b);
    return ANN_OK;
}

int ann_host_alloc(ann_ctx* c, int64_t bytes, void** ptr) {
    if (!c || !ptr) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (bytes < 0) return fail(c, ANN_ERR_ARG, "bytes < 0");
    *ptr = nullptr;
    if (bytes == 0) return ANN_OK;
    ANN_TRY(c, {
        set_device(c);
        ck(cudaMallocHost(ptr, (size_t)bytes), "cudaMallocHost");
    })
}
int ann_host_free(ann_ctx* c, void* ptr) {   // ctx may be NULL (a buffer may outlive its context)
    if (!ptr) return ANN_OK;
    const cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) return fail(c, ANN_ERR_CUDA, std::string("cudaFreeHost: ") + cudaGetErrorString(e));
    return ANN_OK;
}

// ---- inspection
int ann_symm_width(ann_ctx* c, int32_t* w) {
    if (!c || !w) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    *w = c->pot.max_input();
    return ANN_OK;
}
static void download_real_rows(ann_ctx* c, DevBuf& b, double* out, size_t n) {
    if (c->last_prec == ANN_FP64) {
        ck(cudaMemcpyAsync(out, b.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream), "D2H");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
    } else {
        std::vector<float> h(n);
        ck(cudaMemcpyAsync(h.data(), b.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream), "D2H");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        for (size_t k = 0; k < n; ++k) out[k] = h[k];
    }
}
int ann_get_symm(ann_ctx* c, double* G, int64_t cap) {
    if (!c || !G) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        if (cap < (int64_t)c->N * c->pot.max_input()) throw ann_error(ANN_ERR_ARG, "output buffer too small");
        finish_batch(c);
        download_real_rows(c, c->G, G, (size_t)c->N * c->pot.max_input());
    })
}
int ann_get_dedg(ann_ctx* c, double* d, int64_t cap) {
    if (!c || !d) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        if (cap < (int64_t)c->N * c->pot.max_input()) throw ann_error(ANN_ERR_ARG, "output buffer too small");
        finish_batch(c);
        download_real_rows(c, c->dEdG, d, (size_t)c->N * c->pot.max_input());
    })
}
int ann_get_atom_energies(ann_ctx* c, double* e, int64_t cap) {
    if (!c || !e) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        if (cap < (int64_t)c->N) throw ann_error(ANN_ERR_ARG, "output buffer too small");
        finish_batch(c);
        if (c->N > 0) ck(cudaMemcpy(e, c->Eatom.p, sizeof(double) * c->N, cudaMemcpyDeviceToHost), "D2H");
    })
}
int ann_num_neighbors(ann_ctx* c, int64_t* total) {
    if (!c || !total) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        finish_batch(c);
        std::vector<int32_t> nn(c->N);
        if (c->N > 0) ck(cudaMemcpy(nn.data(), c->nn.p, 4 * (size_t)c->N, cudaMemcpyDeviceToHost), "D2H");
        int64_t t = 0;
        for (int v : nn) t += v;
        *total = t;
    })
}
int ann_get_neighbors(ann_ctx* c, int32_t* iout, int32_t* jout, int32_t* img, double* r, int64_t capn) {
    if (!c || !iout || !jout || !img) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_results) throw ann_error(ANN_ERR_STATE, "no computed batch");
        finish_batch(c);
        const size_t N = c->N, cap = c->cap;
        std::vector<int32_t> nn(N), nj(N * cap), ni(N * cap);
        if (N > 0) {
            ck(cudaMemcpy(nn.data(), c->nn.p, 4 * N, cudaMemcpyDeviceToHost), "D2H");
            ck(cudaMemcpy(nj.data(), c->nj.p, 4 * N * cap, cudaMemcpyDeviceToHost), "D2H");
            ck(cudaMemcpy(ni.data(), c->nimg.p, 4 * N * cap, cudaMemcpyDeviceToHost), "D2H");
        }
        std::vector<Vec4d> rr;
        if (r) {
            if (c->last_prec != ANN_FP64) throw ann_error(ANN_ERR_STATE, "pair vectors are only kept in FP64 for FP64 batches");
            rr.resize(N * cap);
            if (N > 0) ck(cudaMemcpy(rr.data(), c->nr.p, sizeof(Vec4d) * N * cap, cudaMemcpyDeviceToHost), "D2H");
        }
        int64_t k = 0;
        for (size_t i = 0; i < N; ++i)
            for (int e = 0; e < nn[i]; ++e) {
                if (k >= capn) throw ann_error(ANN_ERR_CAPACITY, "output arrays too small");
                const int32_t p = ni[i * cap + e];
                iout[k] = (int32_t)i; jout[k] = nj[i * cap + e];
                img[3 * k] = ((int32_t)((uint32_t)p << 22)) >> 22;
                img[3 * k + 1] = ((int32_t)((uint32_t)p << 12)) >> 22;
                img[3 * k + 2] = ((int32_t)((uint32_t)p << 2)) >> 22;
                if (r) { const Vec4d& v = rr[i * cap + e]; r[3 * k] = v.x; r[3 * k + 1] = v.y; r[3 * k + 2] = v.z; }
                ++k;
            }
    })
}

// ---- training
int ann_train_forward(ann_ctx* c, int32_t nstruc, const int64_t* offs, const double* posn, const int32_t* type, const double* cell,
                      const double* Eref, const double* Fref, double wE, double wF, int32_t prec, double* loss3) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (!Eref || !Fref || !loss3) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        leave_md(c);
        upload_batch(c, nstruc, offs, posn, type, cell, false);
        const size_t N = std::max(c->N, 1), S = std::max(c->S, 1), rb = (prec == ANN_FP64) ? 8 : 4;
        c->Eref.ensure(8 * S); c->Fref.ensure(8 * 3 * N); c->loss3.ensure(8 * 4); c->ce.ensure(8 * N);
        c->lam.ensure(rb * 3 * N); c->U.ensure(rb * N * std::max(c->pot.max_input(), 1));
        if (c->S > 0) ck(cudaMemcpyAsync(c->Eref.p, Eref, 8 * (size_t)c->S, cudaMemcpyHostToDevice, c->stream), "H2D Eref");
        if (c->N > 0) ck(cudaMemcpyAsync(c->Fref.p, Fref, 8 * 3 * (size_t)c->N, cudaMemcpyHostToDevice, c->stream), "H2D Fref");
        run_batch(c, prec, true);
        // the loss right behind the E+F sequence, read back with the status word in one round trip;
        // a status that is not clean goes through finish_batch (recover or throw) and the loss again
        auto loss = [&]() {
            ck(cudaMemsetAsync(c->loss3.p, 0, 8 * 4, c->stream), "memset");
            launch_train_loss(c->S, c->N, c->off_d, c->sid.as<int32_t>(), c->Es.as<double>(), c->Fout.as<double>(),
                              c->Eref.as<double>(), c->Fref.as<double>(), wE, wF, c->loss3.as<double>(), c->ce.as<double>(), c->lam.p,
                              prec == ANN_FP64, c->stream);
            ck(cudaGetLastError(), "loss kernel");
            ck(cudaMemcpyAsync(loss3, c->loss3.p, 8 * 3, cudaMemcpyDeviceToHost, c->stream), "D2H loss");
        };
        loss();
        int32_t* sh = status_host(c);
        ck(cudaMemcpyAsync(sh, c->status.p, 4 * 8, cudaMemcpyDeviceToHost, c->stream), "D2H status");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        if (sh[0] != 0) {
            finish_batch(c);
            loss();
            ck(cudaStreamSynchronize(c->stream), "synchronize");
        }
        c->have_train = true; c->train_prec = prec; c->train_wE = wE; c->train_wF = wF;
    })
}
int ann_train_backward(ann_ctx* c, double scale, double* grad, int64_t n) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        set_device(c);
        if (!c->have_train || !c->have_results) throw ann_error(ANN_ERR_STATE, "ann_train_backward needs a preceding ann_train_forward");
        if (n != c->pot.nparams()) throw ann_error(ANN_ERR_ARG, "parameter count mismatch");
        c->grad.ensure(8 * (size_t)std::max<int64_t>(n, 1));
        ck(cudaMemsetAsync(c->grad.p, 0, 8 * (size_t)std::max<int64_t>(n, 1), c->stream), "memset grad");
        const DevPot& pot = c->plan.pot;
        auto go = [&](auto tag) {
            using real = decltype(tag);
            BpArgs<real> b = bp_args<real>(c);
            b.prm = params_of<real>(c->pf, c->pd);
            launch_jvp<real>(pot, b, c->stream);
            MlpArgs<real> m{};
            m.natoms = c->N; m.ntypes = c->pot.ntypes(); m.imax = pot.imax; m.tstart = c->tstart.as<int32_t>(); m.tlist = c->tlist.as<int32_t>();
            m.G = c->G.as<real>(); m.U = c->U.as<real>(); m.ce = c->ce.as<double>(); m.ct = -1.0; m.grad = c->grad.as<double>();
            m.poff = c->poff.as<int32_t>(); m.prm = b.prm;
            launch_mlp_train_grad<real>(pot, m, c->stream);
        };
        if (c->train_prec == ANN_FP64) go(double()); else go(float());
        ck(cudaGetLastError(), "backward kernels");
        if (grad) ck(cudaMemcpyAsync(grad, c->grad.p, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream), "D2H grad");
        int32_t* sh = status_host(c);
        ck(cudaMemcpyAsync(sh, c->status.p, 4 * 8, cudaMemcpyDeviceToHost, c->stream), "D2H status");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        if (sh[0] != 0) throw ann_error(ANN_ERR_CUDA, "device status " + std::to_string(sh[0]) + " in backward pass");
        if (grad) for (int64_t k = 0; k < n; ++k) grad[k] *= scale;
        c->have_grad = true;
    })
}

int ann_adam_init(ann_ctx* c, double lr, double beta1, double beta2, double eps) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        if (!c->have_pot) throw ann_error(ANN_ERR_STATE, "no potential loaded");
        if (!(lr > 0) || !(beta1 >= 0 && beta1 < 1) || !(beta2 >= 0 && beta2 < 1) || !(eps >= 0))
            throw ann_error(ANN_ERR_ARG, "invalid Adam settings (lr > 0, 0 <= beta < 1, eps >= 0)");
        set_device(c);
        const size_t n = (size_t)std::max<int64_t>(c->pot.nparams(), 1);
        c->adam_m.ensure(8 * n); c->adam_v.ensure(8 * n);
        ck(cudaMemsetAsync(c->adam_m.p, 0, 8 * n, c->stream), "memset");
        ck(cudaMemsetAsync(c->adam_v.p, 0, 8 * n, c->stream), "memset");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        c->adam_lr = lr; c->adam_b1 = beta1; c->adam_b2 = beta2; c->adam_eps = eps; c->adam_t = 0;
        c->adam_ready = true;
    })
}
int ann_adam_step(ann_ctx* c, double scale) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        if (!c->adam_ready) throw ann_error(ANN_ERR_STATE, "ann_adam_init first");
        if (!c->have_grad) throw ann_error(ANN_ERR_STATE, "ann_adam_step needs the gradient of a preceding ann_train_backward");
        set_device(c);
        const int64_t n = c->pot.nparams();
        ++c->adam_t;
        const double b1ii = 1.0 / (1.0 - std::pow(c->adam_b1, (double)c->adam_t));
        const double b2ii = 1.0 / (1.0 - std::pow(c->adam_b2, (double)c->adam_t));
        const int64_t before = g_launch_counter;
        launch_adam(n, c->grad.as<double>(), scale, c->adam_m.as<double>(), c->adam_v.as<double>(), c->p64.as<double>(), c->adam_lr, c->adam_b1,
                    c->adam_b2, b1ii, b2ii, c->adam_eps, c->stream);
        launch_param_refresh(n, c->p64.as<double>(), c->pmap.as<int32_t>(), c->pd.w.as<double>(), c->pd.wt.as<double>(), c->pd.b.as<double>(),
                             c->pf.w.as<float>(), c->pf.wt.as<float>(), c->pf.b.as<float>(), c->tc.ok ? c->tcimg.as<uint8_t>() : nullptr,
                             c->stream);
        c->kernels += g_launch_counter - before;
        ck(cudaGetLastError(), "Adam step");
        c->params_dev_newer = true;
        c->have_results = false;
        c->have_grad = false;
    })
}

// ---- molecular dynamics
static void inv3(const double* R, double* Ri) {
    auto at = [&](int r, int c) { return R[3 * c + r]; };
    const double det = at(0, 0) * (at(1, 1) * at(2, 2) - at(1, 2) * at(2, 1)) - at(0, 1) * (at(1, 0) * at(2, 2) - at(1, 2) * at(2, 0)) + at(0, 2) * (at(1, 0) * at(2, 1) - at(1, 1) * at(2, 0));
    if (!(std::fabs(det) > 0)) throw ann_error(ANN_ERR_ARG, "singular cell");
    const double id = 1.0 / det;
    double m[3][3];
    m[0][0] = (at(1, 1) * at(2, 2) - at(1, 2) * at(2, 1)) * id; m[0][1] = (at(0, 2) * at(2, 1) - at(0, 1) * at(2, 2)) * id; m[0][2] = (at(0, 1) * at(1, 2) - at(0, 2) * at(1, 1)) * id;
    m[1][0] = (at(1, 2) * at(2, 0) - at(1, 0) * at(2, 2)) * id; m[1][1] = (at(0, 0) * at(2, 2) - at(0, 2) * at(2, 0)) * id; m[1][2] = (at(0, 2) * at(1, 0) - at(0, 0) * at(1, 2)) * id;
    m[2][0] = (at(1, 0) * at(2, 1) - at(1, 1) * at(2, 0)) * id; m[2][1] = (at(0, 1) * at(2, 0) - at(0, 0) * at(2, 1)) * id; m[2][2] = (at(0, 0) * at(1, 1) - at(0, 1) * at(1, 0)) * id;
    for (int r = 0; r < 3; ++r) for (int cc = 0; cc < 3; ++cc) Ri[3 * cc + r] = m[r][cc];
}

int ann_md_init(ann_ctx* c, int64_t natoms, const double* posn, const double* vel, const int32_t* type, const double* cell,
                const double* mass_t, double dt, double skin, int32_t prec) {
    if (!c || !posn || !vel || !type || !cell || !mass_t) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (dt <= 0 || skin < 0) throw ann_error(ANN_ERR_ARG, "invalid time step or skin");
        c->md_ready = false;
        const int64_t offs[2] = {0, natoms};
        c->md_skin = skin; c->md_dt = dt; c->md_prec = prec;
        c->md_ready = true;  // list cutoff rc + skin from here on
        c->cap = 0;
        upload_batch(c, 1, offs, posn, type, cell, false);
        std::memcpy(c->md_R, cell, sizeof(c->md_R));
        inv3(c->md_R, c->md_Ri);
        c->md_R_d.ensure(72); c->md_Ri_d.ensure(72);
        ck(cudaMemcpy(c->md_R_d.p, c->md_R, 72, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(c->md_Ri_d.p, c->md_Ri, 72, cudaMemcpyHostToDevice), "H2D");
        const int T = c->pot.ntypes();
        c->md_mass_t.assign(mass_t, mass_t + T);
        std::vector<double> minv(T);
        for (int t = 0; t < T; ++t) { if (!(mass_t[t] > 0)) throw ann_error(ANN_ERR_ARG, "masses must be positive"); minv[t] = 1.0 / (mass_t[t] * 103.642696526805); }
        c->minv.ensure(8 * T); c->mass.ensure(8 * T);
        ck(cudaMemcpy(c->minv.p, minv.data(), 8 * T, cudaMemcpyHostToDevice), "H2D");
        ck(cudaMemcpy(c->mass.p, mass_t, 8 * T, cudaMemcpyHostToDevice), "H2D");
        c->vel.ensure(8 * 3 * (size_t)std::max<int64_t>(natoms, 1)); c->disp_ref.ensure(8 * 3 * (size_t)std::max<int64_t>(natoms, 1));
        c->mdflag.ensure(16); c->ke.ensure(16);
        ck(cudaMemcpy(c->vel.p, vel, 8 * 3 * (size_t)natoms, cudaMemcpyHostToDevice), "H2D");
        // initial list + forces
        run_batch(c, prec, true, true);
        finish_batch(c);
        ck(cudaMemcpy(c->disp_ref.p, c->pos.p, 8 * 3 * (size_t)natoms, cudaMemcpyDeviceToDevice), "D2D");
        c->md_rebuilds = 0;
    })
}

int ann_md_run(ann_ctx* c, int32_t nsteps, double* pe, double* ke, int32_t* rebuilds) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        set_device(c);
        if (!c->md_ready) throw ann_error(ANN_ERR_STATE, "ann_md_init first");
        const bool fp64 = c->md_prec == ANN_FP64;
        const double half_skin2 = 0.25 * c->md_skin * c->md_skin;
        int reb = 0;
        for (int step = 0; step < nsteps; ++step) {
            // first half kick + drift + wrap; flags an atom that moved more than skin/2 since the last build
            ck(cudaMemsetAsync(c->mdflag.p, 0, 4, c->stream), "memset");
            launch_md_kick_drift(c->N, c->pos.as<double>(), c->vel.as<double>(), c->F.p, fp64, c->minv.as<double>(), c->type.as<int32_t>(),
                                 c->md_dt, c->md_R_d.as<double>(), c->md_Ri_d.as<double>(), c->disp_ref.as<double>(), c->mdflag.as<int32_t>(),
                                 half_skin2, 0, c->stream);
            int32_t flag = 0;
            ck(cudaMemcpyAsync(&flag, c->mdflag.p, 4, cudaMemcpyDeviceToHost, c->stream), "D2H flag");
            ck(cudaStreamSynchronize(c->stream), "synchronize");
            const bool rebuild = flag != 0;
            if (rebuild) {  // wrap into the cell (Cell::returnToCell) only when the list is rebuilt
                ++reb;
                launch_md_kick_drift(c->N, c->pos.as<double>(), c->vel.as<double>(), c->F.p, fp64, c->minv.as<double>(), c->type.as<int32_t>(),
                                     c->md_dt, c->md_R_d.as<double>(), c->md_Ri_d.as<double>(), c->disp_ref.as<double>(), c->mdflag.as<int32_t>(),
                                     half_skin2, 2, c->stream);
                ck(cudaMemcpyAsync(c->disp_ref.p, c->pos.p, 8 * 3 * (size_t)c->N, cudaMemcpyDeviceToDevice, c->stream), "D2D");
            }
            run_batch(c, c->md_prec, true, rebuild);
            if (rebuild) finish_batch(c);
            // second half kick
            launch_md_kick_drift(c->N, c->pos.as<double>(), c->vel.as<double>(), c->F.p, fp64, c->minv.as<double>(), c->type.as<int32_t>(),
                                 c->md_dt, c->md_R_d.as<double>(), c->md_Ri_d.as<double>(), c->disp_ref.as<double>(), c->mdflag.as<int32_t>(),
                                 half_skin2, 1, c->stream);
        }
        finish_batch(c);
        c->md_rebuilds += reb;
        if (rebuilds) *rebuilds = reb;
        if (pe) ck(cudaMemcpy(pe, c->Es.p, 8, cudaMemcpyDeviceToHost), "D2H pe");
        if (ke) {
            launch_md_ke(c->N, c->vel.as<double>(), c->mass.as<double>(), c->type.as<int32_t>(), c->ke.as<double>(), c->stream);
            ck(cudaMemcpyAsync(ke, c->ke.p, 8, cudaMemcpyDeviceToHost, c->stream), "D2H ke");
            ck(cudaStreamSynchronize(c->stream), "synchronize");
        }
    })
}
int ann_md_get_state(ann_ctx* c, double* posn, double* vel, double* forces) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        set_device(c);
        if (!c->md_ready) throw ann_error(ANN_ERR_STATE, "ann_md_init first");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        if (posn) ck(cudaMemcpy(posn, c->pos.p, 8 * 3 * (size_t)c->N, cudaMemcpyDeviceToHost), "D2H");
        if (vel) ck(cudaMemcpy(vel, c->vel.p, 8 * 3 * (size_t)c->N, cudaMemcpyDeviceToHost), "D2H");
        if (forces) ck(cudaMemcpy(forces, c->Fout.p, 8 * 3 * (size_t)c->N, cudaMemcpyDeviceToHost), "D2H");
    })
}

}  // extern "C"

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

// address of the scratch array on the current device, resolved once per device (the first call
// on a device does it, so that call should come before any stream capture on the device)
static unsigned char* noalloc_scratch(int device) {
    static std::mutex mu;
    static std::map<int, unsigned char*> addr;
    std::lock_guard<std::mutex> g(mu);
    auto it = addr.find(device);
    if (it != addr.end()) return it->second;
    unsigned char* p = nullptr;
    ck(cudaGetSymbolAddress((void**)&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-allocation scratch)");
    addr[device] = p;
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
        unsigned char* s = noalloc_scratch(c->opt.device);
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
                ta.image = c->tcimg.as<uint8_t>(); ta.status = status;
                launch_mlp_tc(c->tc.t[ty], ta, c->tc.smem_bytes(ty), st);
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
