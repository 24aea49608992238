// Test program of include/ann_pair_nn.hpp: drives ann::gpu::PairNN with the arrays a LAMMPS pair
// style receives (x[nall][3], 1-based types, ilist/numneigh/firstneigh with special-bond bits in
// the indices, f[nall][3] accumulated into). Usage: pair_main <potential file> <domain file> <mode>
//   domain file: "nall inum ntypes", then ntypes element names ("NULL" allowed), then per atom
//   "type x y z", then per row "i numneigh j..." (raw LAMMPS indices);
//   mode "nodevice": expects construction to fail with a clear error (no GPU);
//   mode "compute": prints E, the forces added to f (f starts at 1), virial[6] and eatom[nall].
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "ann_pair_nn.hpp"

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::string mode = argv[3];
    if (mode == "nodevice") {
        try {
            ann::gpu::PairNN pair(0, ANN_FP64);
            std::printf("unexpected: created a context\n");
            return 1;
        } catch (std::runtime_error& e) {
            std::printf("error: %s\n", e.what());
            return 0;
        }
    }
    std::ifstream in(argv[2]);
    int nall = 0, inum = 0, ntypes = 0;
    in >> nall >> inum >> ntypes;
    std::vector<std::string> elements(ntypes);
    for (auto& e : elements) in >> e;
    std::vector<double> xs(3 * (size_t)nall), fs(3 * (size_t)nall, 1.0);
    std::vector<int> type(nall);
    for (int i = 0; i < nall; ++i) in >> type[i] >> xs[3 * i] >> xs[3 * i + 1] >> xs[3 * i + 2];
    std::vector<double*> x(nall), f(nall);
    for (int i = 0; i < nall; ++i) { x[i] = &xs[3 * (size_t)i]; f[i] = &fs[3 * (size_t)i]; }
    std::vector<int> ilist(inum), numneigh(nall, 0);
    std::vector<std::vector<int>> rows(nall);
    for (int r = 0; r < inum; ++r) {
        int i = 0, n = 0;
        in >> i >> n;
        ilist[r] = i;
        numneigh[i] = n;
        rows[i].resize(n);
        for (int k = 0; k < n; ++k) in >> rows[i][k];
    }
    std::vector<int*> firstneigh(nall);
    for (int i = 0; i < nall; ++i) firstneigh[i] = rows[i].data();
    ann::gpu::PairNN pair(0, ANN_FP64);
    pair.coeff(argv[1], elements);
    double eng = 0.0, virial[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> eatom(nall, 0.0);
    const double e = pair.compute(inum, ilist.data(), numneigh.data(), firstneigh.data(), nall, x.data(), type.data(), f.data(), &eng,
                                  virial, eatom.data());
    std::printf("%.17g %.17g %.17g\n", e, eng, pair.cutoff());
    for (int i = 0; i < nall; ++i) std::printf("%.17g %.17g %.17g\n", fs[3 * i] - 1.0, fs[3 * i + 1] - 1.0, fs[3 * i + 2] - 1.0);
    std::printf("%.17g %.17g %.17g %.17g %.17g %.17g\n", virial[0], virial[1], virial[2], virial[3], virial[4], virial[5]);
    for (int i = 0; i < nall; ++i) std::printf("%.17g\n", eatom[i]);
    // a second step with the list kept (no reneighbouring): same positions, same energy
    const double e2 = pair.compute(inum, ilist.data(), numneigh.data(), firstneigh.data(), nall, x.data(), type.data(), f.data(),
                                   nullptr, nullptr, nullptr, 0x1FFFFFFF, /*list_changed=*/false);
    std::printf("%.17g\n", e2);
    return 0;
}
