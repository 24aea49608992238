// The caller's neighbour list entry point (ann_compute_list): rows from a full list over local and
// ghost atoms (extlist.cu), then the E+F kernels on those rows.
#include "context.hpp"

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
    b.nsm = c->nsm; b.wait_polls = c->wait_polls;
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
    if (forces) launch_to_double<real>(3 * (size_t)nall, c->lF.as<real>(), c->lFout.as<double>(), c->nsm, st);
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
        if (!fp64) { c->lxh.ensure(16 * (size_t)std::max(nall, 1)); c->lxl.ensure(16 * (size_t)std::max(nall, 1)); }
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
            la.xh = fp64 ? nullptr : c->lxh.as<float4>(); la.xl = fp64 ? nullptr : c->lxl.as<float4>(); la.rc2f = (float)la.rc2;
            la.nsm = c->nsm;
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

}  // extern "C"
