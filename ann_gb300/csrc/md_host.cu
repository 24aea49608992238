// Molecular dynamics entry points: velocity Verlet on the device around the E+F sequence.
#include "context.hpp"

extern "C" {
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

