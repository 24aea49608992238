// Training entry points: input statistics and pre-conditioning of a training set, the
// forward / backward pair of the loss, and the Adam optimiser on the device.
#include "context.hpp"

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

// the loss right behind the E+F sequence, read back with the status word in one round trip; a
// status that is not clean goes through finish_batch (recover or throw) and the loss again. The
// batch, its neighbour rows and its symmetry functions then stay staged for
// ann_train_forward_staged.
static void train_loss(ann_ctx* c, int prec, double wE, double wF, double* loss3) {
    auto loss = [&]() {
        ck(cudaMemsetAsync(c->loss3.p, 0, 8 * 4, c->stream), "memset");
        launch_train_loss(c->S, c->N, c->off_d, c->sid.as<int32_t>(), c->Es.as<double>(), c->Fout.as<double>(),
                          c->Eref.as<double>(), c->Fref.as<double>(), wE, wF, c->train_loss, c->train_norm, c->train_delta,
                          c->loss3.as<double>(), c->ce.as<double>(), c->lam.p, prec == ANN_FP64, c->stream);
        ck(cudaGetLastError(), "loss kernel");
        ck(cudaMemcpyAsync(loss3, c->loss3.p, 8 * 3, cudaMemcpyDeviceToHost, c->stream), "D2H loss");
    };
    loss();
    int32_t* sh = status_host(c);
    ck(cudaMemcpyAsync(sh, c->status.p, 4 * 8, cudaMemcpyDeviceToHost, c->stream), "D2H status");
    ck(cudaStreamSynchronize(c->stream), "synchronize");
    note_rows(c, sh);
    if (sh[0] != 0) {
        finish_batch(c);   // a regrown list is rebuilt from the staged positions
        loss();
        ck(cudaStreamSynchronize(c->stream), "synchronize");
    }
    c->last_loss = loss3[0];
    c->have_train = true; c->train_prec = prec; c->train_wE = wE; c->train_wF = wF;
    c->train_staged = true; c->train_staged_prec = prec;
}

extern "C" {
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
        train_loss(c, prec, wE, wF, loss3);
    })
}
int ann_train_forward_staged(ann_ctx* c, double wE, double wF, int32_t prec, double* loss3) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (!loss3) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        set_device(c);
        if (!c->train_staged)
            throw ann_error(ANN_ERR_STATE, "ann_train_forward_staged needs the batch of a preceding ann_train_forward "
                                           "(no other batch, E+F call, MD step or potential load since)");
        run_staged(c, prec);
        train_loss(c, prec, wE, wF, loss3);
    })
}
int ann_train_set_loss(ann_ctx* c, int32_t loss, int32_t norm, double delta) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (loss < ANN_LOSS_MSE || loss > ANN_LOSS_ASINH) return fail(c, ANN_ERR_ARG, "Invalid loss function.");
    if (norm < ANN_NORM_IDENTITY || norm > ANN_NORM_LOG) return fail(c, ANN_ERR_ARG, "Invalid normalization method.");
    if (!(std::isfinite(delta) && delta > 0.0)) return fail(c, ANN_ERR_ARG, "delta must be finite and > 0");
    c->train_loss = loss; c->train_norm = norm; c->train_delta = delta;
    return ANN_OK;
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
        // the MIXED network pass on the tensor cores (tiles of 128 atoms) when every type fits it,
        // else the SIMT kernel (tiles of 16); either writes per-tile sums added in tile order
        const bool tc_train = c->train_prec == ANN_MIXED && use_tc(c) && c->tct_ok;
        const int tile = tc_train ? TC_M : mlp_train_tile();
        int pstride = 1;
        c->gpart.ensure(mlp_train_part_bytes(pot, c->N, tile, &pstride));
        auto go = [&](auto tag) {
            using real = decltype(tag);
            BpArgs<real> b = bp_args<real>(c);
            b.prm = params_of<real>(c->pf, c->pd);
            launch_jvp<real>(pot, b, c->stream);
            MlpArgs<real> m{};
            m.natoms = c->N; m.ntypes = c->pot.ntypes(); m.imax = pot.imax; m.tstart = c->tstart.as<int32_t>(); m.tlist = c->tlist.as<int32_t>();
            m.G = c->G.as<real>(); m.U = c->U.as<real>(); m.ce = c->ce.as<double>(); m.ct = -1.0; m.grad = c->grad.as<double>();
            m.poff = c->poff.as<int32_t>(); m.prm = b.prm;
            m.gpart = c->gpart.as<double>(); m.pstride = pstride;
            if constexpr (std::is_same<real, float>::value) {
                if (tc_train) {
                    TcTrainArgs ta{};
                    ta.natoms = c->N; ta.imax = pot.imax; ta.ntypes = c->pot.ntypes();
                    ta.tstart = m.tstart; ta.tlist = m.tlist; ta.G = m.G; ta.U = m.U; ta.ce = m.ce; ta.ct = (float)m.ct;
                    ta.image = c->tcimg.as<uint8_t>(); ta.gpart = m.gpart; ta.pstride = pstride;
                    ta.status = c->status.as<int32_t>(); ta.wait_polls = c->wait_polls;
                    launch_mlp_train_tc(c->tc, c->tct, ta, c->stream);
                    launch_grad_blocks(pot, m.tstart, m.poff, m.gpart, pstride, m.grad, TC_M, c->stream);
                    return;
                }
            }
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

}  // extern "C"

// the optimiser of the trainer (opt::algo): state zeroed (RPROP: step sizes 0.1), step counter and
// the running beta powers reset
static void opt_reset(ann_ctx* c, int algo, double lr, double b1, double b2, double eps, double eta, double w) {
    if (!c->have_pot) throw ann_error(ANN_ERR_STATE, "no potential loaded");
    if (algo == OPT_BFGS) throw ann_error(ANN_ERR_UNSUPPORTED, "BFGS keeps a dense P x P matrix; not provided on the device");
    if (algo < OPT_SGD || algo > OPT_CG) throw ann_error(ANN_ERR_ARG, "Invalid optimization algorithm.");
    if (!(lr >= 0) || !(b1 >= 0 && b1 < 1) || !(b2 >= 0 && b2 < 1) || !(eps >= 0) || !(eta >= 0 && eta <= 1) || !(w >= 0 && w <= 1))
        throw ann_error(ANN_ERR_ARG, "invalid optimiser settings (gamma >= 0, 0 <= beta < 1, eps >= 0, 0 <= eta, w <= 1)");
    set_device(c);
    const size_t n = (size_t)std::max<int64_t>(c->pot.nparams(), 1);
    for (DevBuf* b : {&c->opt_s0, &c->opt_s1, &c->opt_s2, &c->opt_gold}) {
        b->ensure(8 * n);
        ck(cudaMemsetAsync(b->p, 0, 8 * n, c->stream), "memset");
    }
    c->opt_part.ensure(8 * 2 * 64 + 8);
    if (algo == OPT_RPROP) {   // RPROP::resize: delta = 0.1 (src/opt/algo.cpp:604-608)
        const std::vector<double> d(n, 0.1);
        ck(cudaMemcpyAsync(c->opt_s0.p, d.data(), 8 * n, cudaMemcpyHostToDevice, c->stream), "H2D");
    }
    ck(cudaStreamSynchronize(c->stream), "synchronize");
    c->opt_algo = algo; c->opt_lr = lr; c->opt_b1 = b1; c->opt_b2 = b2; c->opt_eps = eps; c->opt_eta = eta; c->opt_w = w;
    c->opt_t = 0; c->opt_b1i = b1; c->opt_b2i = b2; c->opt_gamma = lr; c->prev_loss = 0.0;
    c->opt_ready = true;
}

extern "C" {
int ann_opt_init(ann_ctx* c, int32_t algo, double gamma, double eta, double eps, double w) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, { opt_reset(c, algo, gamma, 0.9, 0.999, eps, eta, w); })
}
int ann_adam_init(ann_ctx* c, double lr, double beta1, double beta2, double eps) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        if (!(lr > 0)) throw ann_error(ANN_ERR_ARG, "invalid Adam settings (lr > 0, 0 <= beta < 1, eps >= 0)");
        opt_reset(c, OPT_ADAM, lr, beta1, beta2, eps, 0.0, 0.0);
    })
}
int ann_opt_set_schedule(ann_ctx* c, int32_t decay, double alpha, int32_t period, int32_t reg, double eta) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (decay < ANN_DECAY_CONST || decay > ANN_DECAY_STEP) return fail(c, ANN_ERR_ARG, "Invalid decay schedule.");
    if (reg < ANN_REG_LASSO || reg > ANN_REG_NONE) return fail(c, ANN_ERR_ARG, "Invalid regularization.");
    if (!std::isfinite(alpha) || !std::isfinite(eta)) return fail(c, ANN_ERR_ARG, "alpha and eta must be finite");
    if (decay == ANN_DECAY_STEP && period < 1) return fail(c, ANN_ERR_ARG, "the STEP schedule needs period >= 1");
    c->opt_decay = decay; c->opt_alpha = alpha; c->opt_period = std::max(period, 1); c->opt_reg = reg; c->opt_reg_eta = eta;
    return ANN_OK;
}
int ann_opt_step(ann_ctx* c, double scale) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        if (!c->opt_ready) throw ann_error(ANN_ERR_STATE, "initialise the optimiser first (ann_opt_init / ann_adam_init)");
        if (!c->have_grad) throw ann_error(ANN_ERR_STATE, "an optimiser step needs the gradient of a preceding ann_train_backward");
        set_device(c);
        const int64_t n = c->pot.nparams();
        // the step size of this iteration (Decay::step, opt/decay.cpp:42-62, applied before the
        // optimiser step as nnptefr2.cpp:1025 with the iteration index counted from 0)
        const double t = (double)c->opt_t, al = c->opt_alpha;
        double& gamma = c->opt_gamma;
        switch (c->opt_decay) {
            case ANN_DECAY_EXP: gamma = gamma * (1.0 - al); break;
            case ANN_DECAY_GAUSS: gamma = gamma * (1.0 - 2.0 * al * t); break;
            case ANN_DECAY_SQRT: gamma = gamma * (1.0 - 0.5 * al / (1.0 + al * t)); break;
            case ANN_DECAY_INV: gamma = gamma * (1.0 - al / (1.0 + al * t)); break;
            case ANN_DECAY_STEP: if (c->opt_t > 0 && c->opt_t % c->opt_period == 0) gamma = gamma * al; break;
            default: break;
        }
        OptArgs o{};
        o.n = n; o.algo = c->opt_algo; o.reg = c->opt_reg; o.inc = c->last_loss > c->prev_loss ? 1 : 0;
        o.g = c->grad.as<double>(); o.scale = scale; o.p = c->p64.as<double>();
        o.s0 = c->opt_s0.as<double>(); o.s1 = c->opt_s1.as<double>(); o.s2 = c->opt_s2.as<double>(); o.gold = c->opt_gold.as<double>();
        o.beta = c->opt_part.as<double>() + 2 * 64;
        o.gamma = gamma; o.eta = c->opt_eta; o.eps = c->opt_eps; o.w = c->opt_w; o.b1 = c->opt_b1; o.b2 = c->opt_b2;
        o.b1ii = 1.0 / (1.0 - c->opt_b1i); o.b2ii = 1.0 / (1.0 - c->opt_b2i);
        o.reg_eta = c->opt_reg_eta; o.map = c->pmap.as<int32_t>();
        const int64_t before = g_launch_counter;
        launch_opt(o, c->opt_part.as<double>(), c->stream);
        launch_param_refresh(n, c->p64.as<double>(), c->pmap.as<int32_t>(), c->pd.w.as<double>(), c->pd.wt.as<double>(), c->pd.b.as<double>(),
                             c->pf.w.as<float>(), c->pf.wt.as<float>(), c->pf.b.as<float>(), c->tc.ok ? c->tcimg.as<uint8_t>() : nullptr,
                             c->stream);
        c->kernels += g_launch_counter - before;
        ck(cudaGetLastError(), "optimiser step");
        c->opt_b1i *= c->opt_b1;
        c->opt_b2i *= c->opt_b2;
        ++c->opt_t;
        c->prev_loss = c->last_loss;
        c->params_dev_newer = true;
        c->have_results = false;
        c->have_grad = false;
    })
}
int ann_adam_step(ann_ctx* c, double scale) { return ann_opt_step(c, scale); }

}  // extern "C"
