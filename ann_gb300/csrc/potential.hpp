// Host-side model of a Behler-Parrinello potential in the reference's 'ann' text format.
// Mirrors NNP / NNH / BasisR / BasisA / Cutoff / NN::ANN of the reference (src/nnp/nnp.hpp,
// nnh.hpp, basis_radial.hpp, basis_angular.hpp, cutoff.hpp, src/ml/nn.hpp) as plain data that
// the device plan (plan.cpp) flattens for the kernels.
#pragma once
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace ann {

// enum values follow the reference enums (cutoff.hpp:23-29, basis_radial.hpp:27-35,
// basis_angular.hpp:27-35, nn.hpp:76-103)
enum CutName { CUT_NONE = 0, CUT_STEP = 1, CUT_COS = 2, CUT_TANH = 3, CUT_POLY3 = 4 };
enum RadName { R_NONE = 0, R_GAUSSIAN, R_SECH, R_LOGISTIC, R_TANH, R_LOGCOSH, R_LOGCOSH2 };
enum AngName { A_NONE = 0, A_GAUSS, A_GAUSS2, A_SECH, A_STUDENT3, A_STUDENT4, A_STUDENT5 };
enum Neuron { N_UNKNOWN = 0, N_LINEAR, N_SIGMOID, N_TANH, N_ISRU, N_ARCTAN, N_RELU, N_ELU, N_TANHRE, N_SQRE,
              N_SWISH, N_GELU, N_MISH, N_PFLU, N_SERF, N_LOGISH, N_SOFTPLUS, N_SQPLUS, N_ATISH, N_TEST };

struct ann_error : std::runtime_error {
    int code;
    ann_error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

struct Cutoff {
    int name = CUT_NONE;
    double rc = 0;
};

struct BasisR {                         // basis_radial.hpp
    Cutoff cut;
    int name = R_NONE;
    std::vector<double> rs, eta;
    int size() const { return (int)eta.size(); }
};

struct BasisA {                         // basis_angular.hpp (+ init(), basis_angular.cpp:178-205)
    Cutoff cut;
    int name = A_NONE;
    std::vector<double> eta, zeta;
    std::vector<int> lambda;
    std::vector<int> rflag;             // group of consecutive equal eta (|d|<1e-6)
    std::vector<double> etar;           // eta of each group (first member)
    int size() const { return (int)eta.size(); }
    void init();
};

struct Network {                        // NN::ANN (nn.hpp:243-395)
    int nin = 0;
    std::vector<int> nodes;             // per layer, last = outputs (must be 1 here)
    int neuron = N_UNKNOWN;
    double c = 1.0;
    std::vector<double> inpw, inpb, outw, outb;
    std::vector<std::vector<double>> b; // b[l][n]
    std::vector<std::vector<double>> w; // w[l][n*ni+m] row-major (rows = outputs)
    int nlayer() const { return (int)nodes.size(); }
    int ni(int l) const { return l == 0 ? nin : nodes[l - 1]; }
    int size() const;                   // ANN::size(): biases + weights
    void pack(double* p) const;         // operator>> (nn.cpp:846-859)
    void unpack(const double* p);       // operator<< (nn.cpp:867-880)
};

struct Species {                        // NNH (nnh.hpp) + Type (type.hpp)
    std::string name;
    double mass = 0, energy = 0;
    bool has_mass = false, has_energy = false;
    std::vector<BasisR> R;              // by neighbour type
    std::vector<BasisA> A;              // TensorTri order (tensortri.hpp:194-199)
    std::vector<int> offR, offA;
    int nInputR = 0, nInputA = 0, nInput = 0;
    Network nn;
    void init_input();                  // NNH::init_input (nnh.cpp:94-116)
};

#ifdef __CUDACC__
#define ANN_HD __host__ __device__
#else
#define ANN_HD
#endif
// TensorTri<2> index (src/mem/tensortri.hpp:194-199): angular block of the type pair (i,j)
ANN_HD inline int tri_index(int i, int j) { return (i > j) ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

struct Potential {
    double rc = 0;
    std::vector<Species> sp;
    std::map<std::string, int> index;
    int ntypes() const { return (int)sp.size(); }
    int64_t nparams() const;
    int max_input() const;
    void read_text(const std::string& text);      // NNP::read (nnp.cpp:243-307)
    std::string write_text() const;               // NNP::write (nnp.cpp:197-236)
    void get_params(double* p) const;
    void set_params(const double* p);
    void validate() const;                        // checks the GPU path's supported feature set
};

// ANN::resize initialisation (nn.cpp:1071-1190) of one network's biases and weights
void init_network(Network& nn, int seed, int dist, int init, double sigma_b, double sigma_w);

}  // namespace ann
