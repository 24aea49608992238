// C entry points over the reference's OWN network code (src/ml/nn.cpp), compiled from the
// reference sources by oracle/Makefile, with the plain-loop Eigen stand-in of ref_shim/, into
// oracle/_ref/libref_nn.so.
//
// TEST INFRASTRUCTURE ONLY: tests/golden/make_golden.py and tests/ load it to pin the oracle's
// restatement of the networks. Nothing here is reference source; this file only calls the
// reference classes NN::ANN (resize, operator<< / >>, fpbp2), NN::DODZ, NN::Cost and NN::D2ODZDI.
#include <stdexcept>
#include <string>
#include <vector>
#include "ml/nn.hpp"

static std::string g_err;

extern "C" {

const char* ref_nn_last_error() { return g_err.c_str(); }

// ANN::resize(ANNP, nInp, nodes) with the reference's initialisation (nn.cpp:1019-1190): init
// (NN::Init: 1 RAND, 2 LECUN, 3 HE, 4 XAVIER), neuron (NN::Neuron enum), c, seed, sigma_b / sigma_w
// and dist (rng::dist::Name for both biases and weights)
void* ref_nn_create(int nin, int nlayer, const int* nodes, int neuron, double c, int init, int seed, double sigma_b,
                    double sigma_w, int dist) {
    try {
        NN::ANNP p;
        p.init() = NN::Init((NN::Init::Type)init);
        p.neuron() = NN::Neuron((NN::Neuron::Type)neuron);
        p.c() = c;
        p.seed() = seed;
        p.sigma_b() = sigma_b;
        p.sigma_w() = sigma_w;
        p.dist_b() = rng::dist::Name((rng::dist::Name::Type)dist);
        p.dist_w() = rng::dist::Name((rng::dist::Name::Type)dist);
        NN::ANN* nn = new NN::ANN();
        nn->resize(p, nin, std::vector<int>(nodes, nodes + nlayer));
        return nn;
    } catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void ref_nn_free(void* h) { delete (NN::ANN*)h; }
int ref_nn_size(void* h) { return ((NN::ANN*)h)->size(); }

// parameters in the reference's packing order (operator>> / operator<<, nn.cpp:846-880)
void ref_nn_get_params(void* h, double* out) {
    NN::ANN& nn = *(NN::ANN*)h;
    VecXd v;
    nn >> v;
    for (int k = 0; k < v.size(); ++k) out[k] = v[k];
}
void ref_nn_set_params(void* h, const double* in) {
    NN::ANN& nn = *(NN::ANN*)h;
    VecXd v(nn.size());
    for (int k = 0; k < v.size(); ++k) v[k] = in[k];
    nn << v;
}
void ref_nn_set_scaling(void* h, const double* inpw, const double* inpb, double outw, double outb) {
    NN::ANN& nn = *(NN::ANN*)h;
    for (int m = 0; m < nn.nInp(); ++m) { nn.inpw()[m] = inpw[m]; nn.inpb()[m] = inpb[m]; }
    nn.outw()[0] = outw;
    nn.outb()[0] = outb;
}

// one input through ANN::fpbp2 (nn.cpp:1391-1409), then, for the first output:
//   out      : the network output
//   dodi     : DODZ::grad's dO/dI (nn.cpp:1801-1824), nin values
//   grad     : Cost::grad with dC/dO = 1 (nn.cpp:1712-1770), size() values
//   d2odpdi  : D2ODZDI::grad's d2O/(dp dI) (nn.cpp:2012-2100), size() x nin values (NULL: skipped)
int ref_nn_eval(void* h, const double* inp, double* out, double* dodi, double* grad, double* d2odpdi) {
    try {
        NN::ANN& nn = *(NN::ANN*)h;
        const int nin = nn.nInp(), P = nn.size();
        for (int m = 0; m < nin; ++m) nn.inp()[m] = inp[m];
        nn.fpbp2();
        *out = nn.out()[0];
        NN::DODZ dodz(nn);
        dodz.grad(nn);
        for (int m = 0; m < nin; ++m) dodi[m] = dodz.dodi()(0, m);
        NN::Cost cost(nn);
        VecXd dcdo = VecXd::Constant(nn.nOut(), 1.0);
        const VecXd& g = cost.grad(nn, dcdo);
        for (int k = 0; k < P; ++k) grad[k] = g[k];
        if (d2odpdi) {
            NN::D2ODZDI d2(nn);
            d2.grad(nn);
            for (int k = 0; k < P; ++k)
                for (int m = 0; m < nin; ++m) d2odpdi[(size_t)k * nin + m] = d2.d2odpdi()[k](0, m);
        }
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

}  // extern "C"
