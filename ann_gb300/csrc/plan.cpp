// Builds the flattened device description (DevPot + parameter arrays) of a Potential and decides
// which angular kernel family serves it.
#include "plan_build.hpp"

#include <cmath>
#include <cstring>

#include "../../include/ann_gpu.h"

namespace ann {

static int ilog2_exact(double z) {  // z = 2^k (k in [0,3]) -> k, else -1
    for (int k = 0; k <= 3; ++k) if (z == (double)(1 << k)) return k;
    return -1;
}

void build_plan(const Potential& p, PlanHost& out) {
    p.validate();
    if (p.ntypes() > MAXT) throw ann_error(ANN_ERR_UNSUPPORTED, "more than 4 types are not supported by the GPU path");
    DevPot& d = out.pot;
    std::memset(&d, 0, sizeof(d));
    d.ntypes = p.ntypes();
    d.imax = p.max_input();
    d.rc = p.rc;
    out.rs.clear(); out.reta.clear(); out.aeta.clear(); out.zeta.clear(); out.alam.clear(); out.agrp.clear();
    out.slot2ref.clear(); out.w.clear(); out.wt.clear(); out.b.clear(); out.inpw.clear(); out.inpb.clear();
    const int nt = p.ntypes();
    // ---- fast-path eligibility and damping groups
    bool fast = true;
    int maxg = 1;
    std::vector<std::vector<double>> groups(nt);
    for (int I = 0; I < nt; ++I) {
        const Species& s = p.sp[I];
        for (const BasisA& b : s.A) {
            if (b.size() == 0) continue;
            if (b.name != A_GAUSS) { fast = false; continue; }
            for (int m = 0; m < b.size(); ++m) {
                if (!(b.lambda[m] == 1 || b.lambda[m] == -1) || ilog2_exact(b.zeta[m]) < 0) fast = false;
                const double e = b.etar[b.rflag[m]];
                bool found = false;
                for (double g : groups[I]) if (g == e) found = true;
                if (!found) groups[I].push_back(e);
            }
        }
        if ((int)groups[I].size() > NGMAX) fast = false;
        maxg = std::max(maxg, (int)groups[I].size());
    }
    if (fast) {
        // each (group, k, sign) at most once per block
        for (int I = 0; I < nt && fast; ++I)
            for (const BasisA& b : p.sp[I].A) {
                std::vector<int> used(NGMAX * 8, 0);
                for (int m = 0; m < b.size(); ++m) {
                    int g = 0;
                    for (size_t q = 0; q < groups[I].size(); ++q) if (groups[I][q] == b.etar[b.rflag[m]]) g = (int)q;
                    const int slot = g * 8 + 2 * ilog2_exact(b.zeta[m]) + (b.lambda[m] < 0 ? 1 : 0);
                    if (used[slot]++) fast = false;
                }
            }
    }
    d.fast = fast ? 1 : 0;
    d.fastNG = (maxg <= 1) ? 1 : (maxg <= 2) ? 2 : 4;
    const int S = d.fastNG * 8;
    out.slots = S;
    // ---- per type
    for (int I = 0; I < nt; ++I) {
        const Species& s = p.sp[I];
        DevType& t = d.t[I];
        t.nInput = s.nInput;
        t.nInputR = s.nInputR;
        t.evac = s.energy;
        t.cut = CUT_COS; t.rc = p.rc;
        bool cutset = false;
        for (const BasisR& b : s.R) if (b.size() > 0 && !cutset) { t.cut = b.cut.name; t.rc = b.cut.rc; cutset = true; }
        for (const BasisA& b : s.A) if (b.size() > 0 && !cutset) { t.cut = b.cut.name; t.rc = b.cut.rc; cutset = true; }
        t.ngroups = (int)groups[I].size();
        for (int g = 0; g < t.ngroups && g < NGMAX; ++g) t.ietar2[g] = 1.0 / (groups[I][g] * groups[I][g]);
        for (int J = 0; J < nt; ++J) {
            const BasisR& b = s.R[J];
            DevRadial& r = t.R[J];
            r.name = b.name; r.n = b.size(); r.off = s.offR[J]; r.pidx = (int)out.rs.size();
            for (int m = 0; m < b.size(); ++m) { out.rs.push_back(b.rs[m]); out.reta.push_back(b.eta[m]); }
        }
        for (int blk = 0; blk < nt * (nt + 1) / 2; ++blk) {
            const BasisA& b = s.A[blk];
            DevAngular& a = t.A[blk];
            a.name = b.name; a.n = b.size(); a.off = s.nInputR + s.offA[blk]; a.pidx = (int)out.aeta.size();
            a.sidx = -1;
            for (int m = 0; m < b.size(); ++m) {
                out.aeta.push_back(b.eta[m]); out.zeta.push_back(b.zeta[m]); out.alam.push_back((double)b.lambda[m]);
                int g = 0;
                for (size_t q = 0; q < groups[I].size(); ++q) if (groups[I][q] == b.etar[b.rflag[m]]) g = (int)q;
                out.agrp.push_back(g);
            }
            if (fast && b.size() > 0) {
                a.sidx = (int)out.slot2ref.size();
                std::vector<int> s2r(S, -1);
                for (int m = 0; m < b.size(); ++m) {
                    int g = 0;
                    for (size_t q = 0; q < groups[I].size(); ++q) if (groups[I][q] == b.etar[b.rflag[m]]) g = (int)q;
                    s2r[g * 8 + 2 * ilog2_exact(b.zeta[m]) + (b.lambda[m] < 0 ? 1 : 0)] = m;
                }
                out.slot2ref.insert(out.slot2ref.end(), s2r.begin(), s2r.end());
            }
        }
        // ---- network
        const Network& nn = s.nn;
        if (nn.nlayer() > MAXLAYER) throw ann_error(ANN_ERR_UNSUPPORTED, "networks deeper than 6 weight layers are not supported");
        DevNet& net = t.net;
        net.nlayer = nn.nlayer(); net.nin = nn.nin; net.neuron = nn.neuron; net.c = nn.c;
        net.outw = nn.outw[0]; net.outb = nn.outb[0];
        net.inoff = (int)out.inpw.size();
        out.inpw.insert(out.inpw.end(), nn.inpw.begin(), nn.inpw.end());
        out.inpb.insert(out.inpb.end(), nn.inpb.begin(), nn.inpb.end());
        for (int l = 0; l < nn.nlayer(); ++l) {
            const int no = nn.nodes[l], ni = nn.ni(l);
            net.nodes[l] = no;
            net.woff[l] = (int)out.w.size();
            net.boff[l] = (int)out.b.size();
            out.w.insert(out.w.end(), nn.w[l].begin(), nn.w[l].end());
            for (int m = 0; m < ni; ++m) for (int n = 0; n < no; ++n) out.wt.push_back(nn.w[l][n * ni + m]);
            out.b.insert(out.b.end(), nn.b[l].begin(), nn.b[l].end());
        }
    }
    if (out.slot2ref.empty()) out.slot2ref.push_back(-1);
    auto pad = [](std::vector<double>& v) { if (v.empty()) v.push_back(0.0); };
    pad(out.rs); pad(out.reta); pad(out.aeta); pad(out.zeta); pad(out.alam); pad(out.inpw); pad(out.inpb); pad(out.b); pad(out.w); pad(out.wt);
    if (out.agrp.empty()) out.agrp.push_back(0);
    out.pot.nrad = (int)out.rs.size();
    out.pot.nslot = (int)out.slot2ref.size();
}

}  // namespace ann
