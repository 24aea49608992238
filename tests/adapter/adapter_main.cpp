// Test program of include/ann_nnp.hpp with a minimal Structure type (the accessors the reference's
// Structure offers on this path). Usage: adapter_main <potential file> <xyz-like input> <mode>
//   input: natoms, then 9 cell numbers (R column by column), then per atom "type x y z";
//   mode "nodevice": expects construction to fail with a clear error (no GPU);
//   mode "compute": prints the energy and the forces of NNP::compute and PotNNPE::compute.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "ann_nnp.hpp"

struct Vec3 {
    double v[3] = {0, 0, 0};
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
};
struct Mat3 {
    double m[9] = {0};                       // column-major
    double operator()(int r, int c) const { return m[3 * c + r]; }
};
struct Structure {
    std::vector<Vec3> x, f;
    std::vector<int> t;
    Mat3 R_;
    double pe_ = 0;
    int nAtoms() const { return (int)x.size(); }
    const Vec3& posn(int i) const { return x[i]; }
    Vec3& force(int i) { return f[i]; }
    int type(int i) const { return t[i]; }
    const Mat3& R() const { return R_; }
    double& pe() { return pe_; }
};

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::string mode = argv[3];
    if (mode == "nodevice") {
        try {
            ann::gpu::NNP nnp(0, ANN_FP64);
            std::printf("unexpected: created a context\n");
            return 1;
        } catch (std::runtime_error& e) {
            std::printf("error: %s\n", e.what());
            return 0;
        }
    }
    std::ifstream in(argv[2]);
    int n = 0;
    in >> n;
    Structure s;
    for (int k = 0; k < 9; ++k) in >> s.R_.m[k];
    s.x.resize(n); s.f.resize(n); s.t.resize(n);
    for (int i = 0; i < n; ++i) in >> s.t[i] >> s.x[i][0] >> s.x[i][1] >> s.x[i][2];
    ann::gpu::NNP nnp(0, ANN_FP64);
    ann::gpu::NNP::read(argv[1], nnp);
    const double e = ann::gpu::NNP::compute(nnp, s);
    std::printf("%.15e\n", e);
    for (int i = 0; i < n; ++i) std::printf("%.15e %.15e %.15e\n", s.f[i][0], s.f[i][1], s.f[i][2]);
    ann::gpu::PotNNPE pot(argv[1], 0, ANN_FP64);
    for (auto& v : s.f) v = Vec3();
    s.pe_ = 0;
    const double e2 = pot.compute(s);
    std::printf("%.15e %.15e\n", e2, s.pe_);
    return 0;
}
