// ann_ctx: creation, potentials and parameters, the per-batch kernel sequence with its CUDA-graph
// capture, batch compute and inspection, page-locked host buffers: the core of the extern "C"
// entry points of include/ann_gpu.h. No C++ exception crosses the C boundary.
#include "context.hpp"
#include "transfer.hpp"

static std::mutex g_err_mu;
static std::string g_err;

std::atomic<uint64_t> g_alloc_gen{0};

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

int fail(ann_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    std::lock_guard<std::mutex> g(g_err_mu);
    g_err = m;
    return code;
}
void set_device(ann_ctx* c) { ck(cudaSetDevice(c->opt.device), "cudaSetDevice"); }

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
    for (int k = 0; k < 3; ++k) {
        if (c->gexec[k]) { cudaGraphExecDestroy(c->gexec[k]); c->gexec[k] = nullptr; }
        c->gkey[k] = GraphKey{-1, -1, -1, -1, -1, -1, -1, -1, 0, -1};
    }
}
void drop_graphs(ann_ctx* c) { reset_graph(c); }
void rebuild_plan(ann_ctx* c) {
    build_plan(c->pot, c->plan);
    build_tc_plan(c->plan.pot, c->plan.w, c->plan.b, c->plan.inpw, c->plan.inpb, c->max_smem, c->opt.tc_split, c->tc);
    c->tct_ok = c->tc.ok;
    for (int t = 0; t < c->plan.pot.ntypes && c->tct_ok; ++t) c->tct_ok = plan_tc_train(c->tc.t[t], c->max_smem, c->tct[t]);
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
void sync_params_from_device(ann_ctx* c) {
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
    c->nn.ensure(4 * N); c->ntc.ensure(4 * (size_t)N * T);
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
    c->max_nat = 0;
    c->red_fused = nstruc > 0;
    for (int s = 0; s < nstruc; ++s) {
        c->max_nat = std::max(c->max_nat, c->off_h[s + 1] - c->off_h[s]);
        if (c->off_h[s + 1] == c->off_h[s]) c->red_fused = false;
    }
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
void leave_md(ann_ctx* c) {
    if (!c->md_ready) return;
    c->md_ready = false;
    c->cap = 0;   // re-estimated without the skin
}

void upload_batch(ann_ctx* c, int nstruc, const int64_t* offs, const double* posn, const int32_t* type, const double* cell, bool device_src) {
    if (!c->have_pot) throw ann_error(ANN_ERR_STATE, "no potential loaded");
    // a batch with the offsets of the staged one (a training or MD-like loop) keeps its offset and
    // reduction tables and its per-atom structure index on the device, unless a buffer moved since
    bool same = c->have_batch && offs && nstruc == c->S && c->tables_gen == g_alloc_gen.load() && !c->off_h.empty();
    for (int s = 0; same && s <= nstruc; ++s) same = (offs[s] == (int64_t)c->off_h[s]);
    if (!same) stage_offsets(c, nstruc, offs);
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
    if (c->cap == 0) {
        c->cap = estimate_cap(c, device_src ? nullptr : cell);
    } else if (!c->md_ready && c->opt.max_neighbors <= 0 && c->nn_seen > 0) {
        // rows no longer than 1.25 x the longest seen: the basis and force passes stage rows of
        // cap entries per warp, and a smaller capacity lets more blocks share an SM (a batch with
        // longer rows overflows, regrows the capacity and is computed again)
        const int want = std::max(32, ((int)std::ceil(1.25 * c->nn_seen) + 31) / 32 * 32);
        if (want < c->cap) c->cap = want;
    }
    const uint64_t gen0 = g_alloc_gen.load();
    ensure_batch_buffers(c);
    if (g_alloc_gen.load() != gen0) same = false;
    const cudaMemcpyKind k = device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (!same) {
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
        if (c->N > 0) launch_fill_sid(c->S, c->off_d, c->sid.as<int32_t>(), c->stream);
        c->rarrive.ensure(sizeof(int32_t) * (size_t)std::max(c->S, 1));
        ck(cudaMemsetAsync(c->rarrive.p, 0, sizeof(int32_t) * (size_t)std::max(c->S, 1), c->stream), "memset arrivals");
        c->tables_gen = g_alloc_gen.load();
    }
    // inputs in the library's own page-locked buffers move by one copy kernel, the others by the
    // copy engines
    CopyPlan cp;
    auto put = [&](void* dst, const void* src, size_t bytes, const char* what) {
        if (bytes == 0) return;
        void* v = device_src ? nullptr : host_device_view(src, bytes);
        if (v && cp.add(v, dst, bytes)) return;
        ck(cudaMemcpyAsync(dst, src, bytes, k, c->stream), what);
    };
    put(c->pos.p, posn, sizeof(double) * 3 * (size_t)c->N, "copy positions");
    put(c->type.p, type, sizeof(int32_t) * (size_t)c->N, "copy types");
    put(c->cell.p, cell, sizeof(double) * 9 * (size_t)c->S, "copy cells");
    launch_copy_plan(cp, c->nsm, c->stream);
    c->have_batch = true;
    c->have_results = false;
    c->train_staged = false;
}

// ---------------------------------------------------------------- the E+F kernel sequence
static NbrArgs nbr_args(ann_ctx* c, double rc) {
    NbrArgs a{};
    a.nstruc = c->S; a.natoms = c->N; a.ntypes = c->pot.ntypes(); a.cap = c->cap; a.rc = rc;
    a.off = c->off_d; a.cell = c->cell.as<double>(); a.pos = c->pos.as<double>(); a.type = c->type.as<int32_t>(); a.sid = c->sid.as<int32_t>();
    a.grid_per_sm = c->tune_nbr;
    a.nsm = c->nsm;
    a.max_nat = c->max_nat;
    a.geo = c->geo.as<StrucGeo>(); a.pos4 = c->pos4.as<float4>(); a.abin = c->abin.as<int32_t>(); a.abc = c->abc.as<int32_t>(); a.am = c->am.as<int32_t>();
    a.aslot = c->aslot.as<int32_t>(); a.bcount = c->bcount.as<int32_t>(); a.bstart = c->bstart.as<int32_t>(); a.bidx = c->bidx.as<int32_t>();
    a.bm = c->bm.as<int32_t>(); a.bpos4 = c->bpos4.as<float4>(); a.bposd = c->bposd.as<double>(); a.nbins_cap = c->nbins_cap;
    a.nn = c->nn.as<int32_t>(); a.ntc = c->ntc.as<int32_t>(); a.nj = c->nj.as<int32_t>();
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
    t.arrive = c->red_fused ? c->rarrive.as<int32_t>() : nullptr;
    return t;
}



template <typename real>
static void enqueue_ef(ann_ctx* c, bool forces, int mode) {
    cudaStream_t st = c->stream;
    ck(cudaMemsetAsync(c->status.p, 0, 4 * 8, st), "memset status");   // part of the captured sequence
    const bool fp64 = std::is_same<real, double>::value;
    const DevPot& pot = c->plan.pot;
    BpArgs<real> b = bp_args<real>(c);
    b.prm = params_of<real>(c->pf, c->pd);
    if (mode == SEQ_STAGED) {
        // neighbour rows, type lists and symmetry functions of the staged batch are on the device
        mark(c, 0); mark(c, 1); mark(c, 2); mark(c, 3);
    } else {
    const bool build_list = (mode == SEQ_BUILD);
    // the per-type atom lists depend on the types only: outside the phase-timed and debug modes
    // they run on a side stream that forks here and joins before the networks (a parallel branch
    // of the captured graph, beside the neighbour search and the symmetry functions)
    const bool side = !c->profile && !c->debug;
    auto type_lists = [&](cudaStream_t s) {
        launch_type_lists(c->N, c->pot.ntypes(), c->type.as<int32_t>(), c->tcount.as<int32_t>(), c->tstart.as<int32_t>(),
                          c->tlist.as<int32_t>(), c->status.as<int32_t>(), s);
    };
    // the side branch also clears the G rows for the symmetry pass, off the critical path
    if (side) {
        ck(cudaEventRecord(c->ev_fork, st), "event record");
        ck(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "stream wait");
        type_lists(c->side);
        if (c->N > 0) launch_zero_rows<real>(c->G.as<real>(), (size_t)c->N * pot.imax, c->side);
        ck(cudaEventRecord(c->ev_join, c->side), "event record");
        b.out_zeroed = 1;
    }
    mark(c, 0);
    // MD: the list holds rc + skin and is rebuilt only when an atom moved skin/2; between
    // rebuilds its pair vectors are recomputed from the current positions
    if (!build_list && !c->md_ready) throw ann_error(ANN_ERR_STATE, "a list refresh outside MD");
    if (build_list) launch_neighbors(nbr_args(c, c->pot.rc + (c->md_ready ? c->md_skin : 0.0)), fp64, st);
    else launch_refresh_geometry(nbr_args(c, c->pot.rc + c->md_skin), fp64, st);
    check_phase(c, "neighbour list");
    mark(c, 1);
    if (!side) type_lists(st);
    check_phase(c, "type lists");
    mark(c, 2);
    if (side) ck(cudaStreamWaitEvent(st, c->ev_join, 0), "stream wait");
    launch_symm<real>(pot, b, st);
    check_phase(c, "symmetry functions");
    mark(c, 3);
    b.out_zeroed = 0;
    }
    enqueue_networks<real>(c, c->N, c->G, c->dEdG, c->Eatom, c->tstart, c->tlist, b.prm);
    check_phase(c, "networks");
    mark(c, 4);
    if (forces) {
        // the symmetry pass clears F atom by atom; the staged sequence runs no symmetry pass
        if (mode == SEQ_STAGED) cudaMemsetAsync(c->F.p, 0, sizeof(real) * 3 * (size_t)std::max(c->N, 1), st);
        launch_force<real>(pot, b, st);
    }
    check_phase(c, "forces");
    mark(c, 5);
    launch_reduce_structures<real>(c->S, red_table(c), c->Eatom.as<double>(), forces ? c->W.as<real>() : nullptr,
                                   c->F.as<real>(), c->Es.as<double>(), c->Ws.as<double>(), forces ? c->Fout.as<double>() : nullptr, st);
    check_phase(c, "reductions");
    mark(c, 6);
}

static void run_sequence(ann_ctx* c, int prec, bool forces, int mode) {
    if (!c->have_batch) throw ann_error(ANN_ERR_STATE, "no batch staged");
    if (prec != ANN_FP64 && prec != ANN_MIXED) throw ann_error(ANN_ERR_ARG, "invalid precision");
    // shared-memory needs of this batch (neighbour rows are staged per warp)
    const size_t need_bp = bp_smem_bytes(c->plan.pot, c->cap, prec == ANN_FP64) + 1024;
    const size_t need_mlp = mlp_smem_bytes(c->plan.pot, prec == ANN_FP64, false) + 1024;
    if (mode == SEQ_BUILD && nbr_smem_bytes(c->cap, prec == ANN_FP64) + 1024 > (size_t)c->max_smem)
        throw ann_error(ANN_ERR_CAPACITY, "neighbour capacity " + std::to_string(c->cap) + " exceeds the neighbour search's shared memory");
    if (need_bp > (size_t)c->max_smem)
        throw ann_error(ANN_ERR_CAPACITY, "neighbour capacity " + std::to_string(c->cap) + " needs " + std::to_string(need_bp) +
                                              " B of shared memory per block (device limit " + std::to_string(c->max_smem) + ")");
    if (!(prec == ANN_MIXED && use_tc(c)) && need_mlp > (size_t)c->max_smem)
        throw ann_error(ANN_ERR_UNSUPPORTED, "networks too wide for the shared-memory network kernel");
    const GraphKey key{c->S, c->N, c->cap, prec, forces ? 1 : 0, c->nbins_cap, (int)(c->rchunk_h.size() / 3), c->md_ready ? 1 : 0, g_alloc_gen.load(),
                       (nbr_local_binning(c->max_nat) ? 1 : 0) | (c->red_fused ? 2 : 0)};
    const bool graphs = c->opt.use_graphs && c->N > 0 && !c->profile;
    const int gs = mode;
    if (graphs) {
        if (!(c->gexec[gs] && c->gkey[gs] == key)) {
            if (c->gexec[gs]) { cudaGraphExecDestroy(c->gexec[gs]); c->gexec[gs] = nullptr; }
            cudaGraph_t g = nullptr;
            const int64_t before = g_launch_counter;
            ck(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            if (prec == ANN_FP64) enqueue_ef<double>(c, forces, mode); else enqueue_ef<float>(c, forces, mode);
            const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
            if (ce != cudaSuccess) {
                // locate the failing launch: replay the sequence eagerly with per-phase checks
                cudaGetLastError();
                if (g) cudaGraphDestroy(g);
                const bool d0 = c->debug;
                c->debug = true;
                try {
                    if (prec == ANN_FP64) enqueue_ef<double>(c, forces, mode); else enqueue_ef<float>(c, forces, mode);
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
        if (prec == ANN_FP64) enqueue_ef<double>(c, forces, mode); else enqueue_ef<float>(c, forces, mode);
        c->kernels += g_launch_counter - before;
    }
    ck(cudaGetLastError(), "kernel launch");
    c->last_prec = prec;
    c->have_results = true;
    c->have_forces = forces;
}

void run_batch(ann_ctx* c, int prec, bool forces, bool build_list) {
    c->train_staged = false;
    run_sequence(c, prec, forces, build_list ? SEQ_BUILD : SEQ_REFRESH);
}

void run_staged(ann_ctx* c, int prec) {
    if (!c->train_staged) throw ann_error(ANN_ERR_STATE, "no staged training batch");
    if (prec != c->train_staged_prec)
        throw ann_error(ANN_ERR_STATE, "the staged symmetry functions were computed in the other precision");
    run_sequence(c, prec, true, SEQ_STAGED);
}

// a page-locked copy of the device status word, for reads that ride along with result copies
int32_t* status_host(ann_ctx* c) {
    if (!c->status_h) {
        ck(cudaMallocHost(reinterpret_cast<void**>(&c->status_h), 4 * 8), "cudaMallocHost status");
        host_register(c->status_h, 4 * 8);
    }
    return c->status_h;
}

// wait for the batch; on neighbour overflow grow the capacity and recompute
void finish_batch(ann_ctx* c) {
    for (int attempt = 0; attempt < 6; ++attempt) {
        int32_t st[8];
        ck(cudaMemcpyAsync(st, c->status.p, sizeof(st), cudaMemcpyDeviceToHost, c->stream), "D2H status");
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        note_rows(c, st);
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
    o->tc_groups = 0; o->tc_split = 0;
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
        ck(cudaEventCreateWithFlags(&c->ev_net_fork, cudaEventDisableTiming), "event create");
        ck(cudaEventCreateWithFlags(&c->ev_net_join, cudaEventDisableTiming), "event create");
        configure_kernels();
        cudaDeviceGetAttribute(&c->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->opt.device);
        cudaDeviceGetAttribute(&c->tc.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->opt.device);
        ck(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->opt.device), "SM count");
        if (c->nsm < 1) c->nsm = 1;
        if (c->opt.mlp_backend < 0 || c->opt.mlp_backend > 2) throw ann_error(ANN_ERR_ARG, "mlp_backend must be 0, 1 or 2");
        if (c->opt.tc_groups != 0 && c->opt.tc_groups != 1 && c->opt.tc_groups != 2 && c->opt.tc_groups != 4)
            throw ann_error(ANN_ERR_ARG, "tc_groups must be 0, 1, 2 or 4");
        if (c->opt.tc_split < 0 || c->opt.tc_split > 3) throw ann_error(ANN_ERR_ARG, "tc_split must be 0, 1, 2 or 3");
        const char* dbg = std::getenv("ANN_DEBUG");
        c->debug = dbg && dbg[0] == '1';
        if (c->debug) c->opt.use_graphs = 0;
    } catch (ann_error& e) {
        if (c->stream) cudaStreamDestroy(c->stream);
        if (c->side) cudaStreamDestroy(c->side);
        if (c->ev_fork) cudaEventDestroy(c->ev_fork);
        if (c->ev_join) cudaEventDestroy(c->ev_join);
        if (c->ev_net_fork) cudaEventDestroy(c->ev_net_fork);
        if (c->ev_net_join) cudaEventDestroy(c->ev_net_join);
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
                      &c->bcount, &c->bstart, &c->bidx, &c->bm, &c->bpos4, &c->bposd, &c->nn, &c->ntc, &c->nj, &c->nimg,
                      &c->nr, &c->scan_tmp, &c->counter, &c->status, &c->G, &c->dEdG, &c->Eatom, &c->F, &c->W, &c->Es, &c->Ws, &c->Fout,
                      &c->tcount, &c->tstart, &c->tlist, &c->Eref, &c->Fref, &c->loss3, &c->ce, &c->lam, &c->U, &c->grad, &c->gpart,
                      &c->vel, &c->minv, &c->mass, &c->disp_ref, &c->mdflag, &c->ke, &c->md_R_d, &c->md_Ri_d,
                      &c->tables, &c->rpartial, &c->rarrive, &c->tcimg, &c->p64, &c->pmap, &c->opt_s0, &c->opt_s1, &c->opt_s2, &c->opt_gold, &c->opt_part,
                      &c->lx, &c->ltype, &c->lilist, &c->lnoff, &c->lneigh, &c->lrtype, &c->lnn, &c->lntc, &c->lnj, &c->lnr, &c->lG,
                      &c->ldEdG, &c->lEatom, &c->lF, &c->lW, &c->lFout, &c->ltcount, &c->ltstart, &c->ltlist, &c->ltables, &c->lpartial,
                      &c->lEs, &c->lWs, &c->st_acc, &c->st_n, &c->st_part, &c->st_pcount})
        b->release();
    for (auto& e : c->ev) if (e) cudaEventDestroy(e);
    if (c->status_h) { host_unregister(c->status_h); cudaFreeHost(c->status_h); }
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_net_fork) cudaEventDestroy(c->ev_net_fork);
    if (c->ev_net_join) cudaEventDestroy(c->ev_net_join);
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
        c->opt_ready = false;
        c->st_ready = false;   // statistics belong to the previous potential's inputs
        c->train_staged = false;   // so do the staged training batch's symmetry functions
        c->nn_seen = 0;            // and the row lengths (the cutoff may differ)
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
int ann_network_form(ann_ctx* c, int32_t t, int32_t* backend, int32_t* split) {
    if (!c || !backend || !split) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (!c->have_pot) return fail(c, ANN_ERR_STATE, "no potential loaded");
    if (t < 0 || t >= c->pot.ntypes()) return fail(c, ANN_ERR_ARG, "type index out of range");
    const bool tc = use_tc(c);
    *backend = tc ? 2 : 1;
    *split = tc ? c->tc.t[t].split : 0;
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
        // results into the library's own page-locked buffers move by one copy kernel (with the
        // status word), the others by the copy engines
        int32_t* sh = status_host(c);
        auto copy_out = [&](bool with_status) {
            CopyPlan cp;
            auto get = [&](void* dst, const void* src, size_t bytes, const char* what) {
                if (bytes == 0) return;
                void* v = host_device_view(dst, bytes);
                if (v && cp.add(src, v, bytes)) return;
                ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream), what);
            };
            get(energy, c->Es.p, sizeof(double) * c->S, "D2H energy");
            if (forces) get(forces, c->Fout.p, sizeof(double) * 3 * (size_t)c->N, "D2H forces");
            if (virial) get(virial, c->Ws.p, sizeof(double) * 9 * (size_t)c->S, "D2H virial");
            if (with_status) get(sh, c->status.p, 4 * 8, "D2H status");
            launch_copy_plan(cp, c->nsm, c->stream);
            ck(cudaGetLastError(), "copy kernel");
        };
        copy_out(true);
        ck(cudaStreamSynchronize(c->stream), "synchronize");
        note_rows(c, sh);
        if (sh[0] != 0) {
            finish_batch(c);
            copy_out(false);
            ck(cudaStreamSynchronize(c->stream), "synchronize");
        }
    })
}

}  // extern "C"


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

extern "C" {
int ann_host_alloc(ann_ctx* c, int64_t bytes, void** ptr) {
    if (!c || !ptr) return fail(c, ANN_ERR_ARG, "NULL argument");
    if (bytes < 0) return fail(c, ANN_ERR_ARG, "bytes < 0");
    *ptr = nullptr;
    if (bytes == 0) return ANN_OK;
    ANN_TRY(c, {
        set_device(c);
        ck(cudaMallocHost(ptr, (size_t)bytes), "cudaMallocHost");
        host_register(*ptr, (size_t)bytes);
    })
}
int ann_host_free(ann_ctx* c, void* ptr) {   // ctx may be NULL (a buffer may outlive its context)
    if (!ptr) return ANN_OK;
    host_unregister(ptr);
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

}  // extern "C"
