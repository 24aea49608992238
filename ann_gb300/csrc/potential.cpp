// Reader / writer of the reference 'ann' potential format and parameter packing.
#include "potential.hpp"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <sstream>

#include "../../include/ann_gpu.h"

namespace ann {

// ------------------------------------------------------------------ BasisA::init (basis_angular.cpp:178-205)
void BasisA::init() {
    const int n = size();
    rflag.assign(n, 0);
    etar.clear();
    if (n == 0) return;
    int flag = 0;
    etar.push_back(eta[0]);
    for (int i = 1; i < n; ++i) {
        if (std::fabs(eta[i] - eta[i - 1]) < 1.0e-6) rflag[i] = flag;
        else { rflag[i] = ++flag; etar.push_back(eta[i]); }
    }
}

// ------------------------------------------------------------------ Network
int Network::size() const {
    int s = 0;
    for (int l = 0; l < nlayer(); ++l) s += nodes[l] + nodes[l] * ni(l);
    return s;
}
void Network::pack(double* p) const {
    int c = 0;
    for (int l = 0; l < nlayer(); ++l) for (int n = 0; n < nodes[l]; ++n) p[c++] = b[l][n];
    for (int l = 0; l < nlayer(); ++l) { const int k = ni(l); for (int m = 0; m < k; ++m) for (int n = 0; n < nodes[l]; ++n) p[c++] = w[l][n * k + m]; }
}
void Network::unpack(const double* p) {
    int c = 0;
    for (int l = 0; l < nlayer(); ++l) for (int n = 0; n < nodes[l]; ++n) b[l][n] = p[c++];
    for (int l = 0; l < nlayer(); ++l) { const int k = ni(l); for (int m = 0; m < k; ++m) for (int n = 0; n < nodes[l]; ++n) w[l][n * k + m] = p[c++]; }
}

// ------------------------------------------------------------------ Species
void Species::init_input() {
    nInputR = 0; offR.assign(R.size(), 0);
    for (size_t i = 0; i < R.size(); ++i) { nInputR += R[i].size(); offR[i] = (i == 0) ? 0 : offR[i - 1] + R[i - 1].size(); }
    nInputA = 0; offA.assign(A.size(), 0);
    for (size_t i = 0; i < A.size(); ++i) { nInputA += A[i].size(); offA[i] = (i == 0) ? 0 : offA[i - 1] + A[i - 1].size(); }
    nInput = nInputR + nInputA;
}

// ------------------------------------------------------------------ Potential
int64_t Potential::nparams() const { int64_t s = 0; for (auto& x : sp) s += x.nn.size(); return s; }
int Potential::max_input() const { int m = 0; for (auto& x : sp) m = std::max(m, x.nInput); return m; }
void Potential::get_params(double* p) const { int64_t c = 0; for (auto& x : sp) { x.nn.pack(p + c); c += x.nn.size(); } }
void Potential::set_params(const double* p) { int64_t c = 0; for (auto& x : sp) { x.nn.unpack(p + c); c += x.nn.size(); } }

namespace {
struct Lines {
    std::vector<std::vector<std::string>> v;
    size_t pos = 0;
    explicit Lines(const std::string& text) {
        std::istringstream is(text);
        std::string line;
        while (std::getline(is, line)) {
            std::vector<std::string> toks;
            std::istringstream ls(line);
            std::string t;
            while (ls >> t) toks.push_back(t);
            v.push_back(toks);
        }
    }
    const std::vector<std::string>& next() {
        if (pos >= v.size()) throw ann_error(ANN_ERR_FORMAT, "potential file: unexpected end of file at line " + std::to_string(pos + 1));
        return v[pos++];
    }
    int line() const { return (int)pos; }
};
const std::string& tok(const Lines& L, const std::vector<std::string>& l, size_t i) {
    if (i >= l.size()) throw ann_error(ANN_ERR_FORMAT, "potential file: missing field on line " + std::to_string(L.line()));
    return l[i];
}
double num(const Lines& L, const std::vector<std::string>& l, size_t i) {
    const std::string& s = tok(L, l, i);
    char* end = nullptr;
    const double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str()) throw ann_error(ANN_ERR_FORMAT, "potential file: bad number '" + s + "' on line " + std::to_string(L.line()));
    return v;
}
int cut_read(const std::string& s) {  // Cutoff::Name::read (cutoff.cpp:15-21)
    if (s == "STEP") return CUT_STEP; if (s == "COS") return CUT_COS; if (s == "TANH") return CUT_TANH; if (s == "POLY3") return CUT_POLY3;
    throw ann_error(ANN_ERR_FORMAT, "invalid cutoff name '" + s + "'");
}
const char* cut_name(int n) { switch (n) { case CUT_STEP: return "STEP"; case CUT_COS: return "COS"; case CUT_TANH: return "TANH"; case CUT_POLY3: return "POLY3"; default: return "NONE"; } }
int radial_read(const std::string& s) {  // BasisR::Name::read (basis_radial.cpp:25-33)
    if (s == "GAUSSIAN") return R_GAUSSIAN; if (s == "SECH") return R_SECH; if (s == "LOGISTIC") return R_LOGISTIC;
    if (s == "TANH") return R_TANH; if (s == "LOGCOSH") return R_LOGCOSH; if (s == "LOGCOSH2") return R_LOGCOSH2;
    throw ann_error(ANN_ERR_FORMAT, "invalid radial function '" + s + "'");
}
const char* radial_name(int n) { static const char* v[] = {"NONE", "GAUSSIAN", "SECH", "LOGISTIC", "TANH", "LOGCOSH", "LOGCOSH2"}; return (n >= 0 && n < 7) ? v[n] : "NONE"; }
int angular_read(const std::string& s) {  // BasisA::Name::read (basis_angular.cpp:24-32)
    if (s == "GAUSS") return A_GAUSS; if (s == "GAUSS2") return A_GAUSS2; if (s == "SECH") return A_SECH;
    if (s == "STUDENT3") return A_STUDENT3; if (s == "STUDENT4") return A_STUDENT4; if (s == "STUDENT5") return A_STUDENT5;
    throw ann_error(ANN_ERR_FORMAT, "invalid angular function '" + s + "'");
}
const char* angular_name(int n) { static const char* v[] = {"NONE", "GAUSS", "GAUSS2", "SECH", "STUDENT3", "STUDENT4", "STUDENT5"}; return (n >= 0 && n < 7) ? v[n] : "NONE"; }
const char* neuron_names[] = {"UNKNOWN", "LINEAR", "SIGMOID", "TANH", "ISRU", "ARCTAN", "RELU", "ELU", "TANHRE", "SQRE",
                              "SWISH", "GELU", "MISH", "PFLU", "SERF", "LOGISH", "SOFTPLUS", "SQPLUS", "ATISH", "TEST"};
int neuron_read(const std::string& s) {  // Neuron::read (nn.cpp:120-140)
    for (int i = 1; i < 20; ++i) if (s == neuron_names[i]) return i;
    return N_UNKNOWN;
}

void read_cutoff(Lines& L, const std::vector<std::string>& hd, Cutoff& c) {
    c.name = cut_read(tok(L, hd, 1));
    c.rc = num(L, hd, 2);
    if (c.rc < 0) throw ann_error(ANN_ERR_FORMAT, "invalid cutoff distance");  // cutoff.cpp:52
}
void read_basisR(Lines& L, BasisR& b) {  // BasisR::read (basis_radial.cpp:123-143)
    const auto& hd = L.next();
    if (tok(L, hd, 0) != "BasisR") throw ann_error(ANN_ERR_FORMAT, "expected 'BasisR' on line " + std::to_string(L.line()));
    read_cutoff(L, hd, b.cut);
    b.name = radial_read(tok(L, hd, 3));
    const int n = (int)num(L, hd, 4);
    if (n < 0) throw ann_error(ANN_ERR_FORMAT, "invalid number of functions");
    b.rs.assign(n, 0); b.eta.assign(n, 0);
    for (int i = 0; i < n; ++i) { const auto& l = L.next(); b.rs[i] = num(L, l, 0); b.eta[i] = num(L, l, 1); }
}
void read_basisA(Lines& L, BasisA& b) {  // BasisA::read (basis_angular.cpp:116-138)
    const auto& hd = L.next();
    if (tok(L, hd, 0) != "BasisA") throw ann_error(ANN_ERR_FORMAT, "expected 'BasisA' on line " + std::to_string(L.line()));
    read_cutoff(L, hd, b.cut);
    b.name = angular_read(tok(L, hd, 3));
    const int n = (int)num(L, hd, 4);
    if (n < 0) throw ann_error(ANN_ERR_FORMAT, "invalid number of functions");
    b.eta.assign(n, 0); b.zeta.assign(n, 0); b.lambda.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        const auto& l = L.next();
        b.eta[i] = num(L, l, 0); b.zeta[i] = num(L, l, 1); b.lambda[i] = std::atoi(tok(L, l, 2).c_str());
    }
    b.init();
}
void read_network(Lines& L, Network& nn) {  // ANN::read (nn.cpp:1495-1578)
    const auto& cfg = L.next();
    std::vector<int> nodes;
    for (size_t i = 1; i < cfg.size(); ++i) nodes.push_back(std::atoi(cfg[i].c_str()));
    if (nodes.size() < 2) throw ann_error(ANN_ERR_FORMAT, "invalid network configuration on line " + std::to_string(L.line()));
    for (int n : nodes) if (n <= 0) throw ann_error(ANN_ERR_FORMAT, "invalid layer size");  // nn.cpp:1083-1085
    nn.nin = nodes[0];
    nn.nodes.assign(nodes.begin() + 1, nodes.end());
    const auto& ne = L.next();
    nn.neuron = neuron_read(tok(L, ne, 1));
    nn.c = num(L, ne, 2);
    if (nn.neuron == N_UNKNOWN) throw ann_error(ANN_ERR_FORMAT, "invalid neuron '" + tok(L, ne, 1) + "'");
    const int nout = nn.nodes.back();
    auto readvec = [&](std::vector<double>& v, int n) {
        const auto& l = L.next();
        v.assign(n, 0);
        for (int i = 0; i < n; ++i) v[i] = num(L, l, i + 1);
    };
    readvec(nn.inpw, nn.nin); readvec(nn.outw, nout); readvec(nn.inpb, nn.nin); readvec(nn.outb, nout);
    nn.b.resize(nn.nlayer()); nn.w.resize(nn.nlayer());
    for (int l = 0; l < nn.nlayer(); ++l) readvec(nn.b[l], nn.nodes[l]);
    for (int l = 0; l < nn.nlayer(); ++l) readvec(nn.w[l], nn.nodes[l] * nn.ni(l));  // row-major on file (nn.cpp:1465-1473)
}
}  // namespace

void Potential::read_text(const std::string& text) {
    Lines L(text);
    L.next();  // header
    const auto& nt_l = L.next();
    const int nt = (int)num(L, nt_l, 1);
    if (nt <= 0) throw ann_error(ANN_ERR_FORMAT, "invalid number of types");  // nnp.cpp:253
    sp.assign(nt, Species());
    index.clear();
    for (int n = 0; n < nt; ++n) {  // Type::read (type.cpp:35-80)
        const auto& l = L.next();
        for (size_t i = 0; i + 1 < l.size(); i += 2) {
            std::string tag = l[i];
            for (auto& ch : tag) ch = (char)std::toupper((unsigned char)ch);
            if (tag == "NAME") sp[n].name = l[i + 1];
            else if (tag == "MASS") { sp[n].mass = std::atof(l[i + 1].c_str()); sp[n].has_mass = true; }
            else if (tag == "ENERGY") { sp[n].energy = std::atof(l[i + 1].c_str()); sp[n].has_energy = true; }
        }
        if (sp[n].name.empty()) throw ann_error(ANN_ERR_FORMAT, "type without a name on line " + std::to_string(L.line()));
        index[sp[n].name] = n;
    }
    rc = num(L, L.next(), 1);
    if (rc <= 0) throw ann_error(ANN_ERR_FORMAT, "invalid cutoff");  // nnp.cpp:264
    for (auto& x : sp) { x.R.assign(nt, BasisR()); x.A.assign(nt * (nt + 1) / 2, BasisA()); }
    auto idx = [&](const std::string& s) {
        auto it = index.find(s);
        if (it == index.end()) throw ann_error(ANN_ERR_FORMAT, "unknown type name '" + s + "'");
        return it->second;
    };
    for (int i = 0; i < nt; ++i) {
        const int II = idx(tok(L, L.next(), 1));
        for (int j = 0; j < nt; ++j) { const int JJ = idx(tok(L, L.next(), 1)); read_basisR(L, sp[II].R[JJ]); }
        for (int j = 0; j < nt; ++j) for (int k = j; k < nt; ++k) {
            const auto& l = L.next();
            const int JJ = idx(tok(L, l, 1)), KK = idx(tok(L, l, 2));
            read_basisA(L, sp[II].A[tri_index(JJ, KK)]);
        }
    }
    for (auto& x : sp) x.init_input();
    for (int n = 0; n < nt; ++n) {
        const int II = idx(tok(L, L.next(), 1));
        read_network(L, sp[II].nn);
        if (sp[II].nn.nin != sp[II].nInput)
            throw ann_error(ANN_ERR_FORMAT, "network of type " + sp[II].name + " has " + std::to_string(sp[II].nn.nin) +
                                                " inputs but its basis defines " + std::to_string(sp[II].nInput));
    }
}

std::string Potential::write_text() const {  // NNP::write (nnp.cpp:197-236), formats as the reference
    std::string out;
    char buf[256];
    auto put = [&](const char* fmt, auto... a) { std::snprintf(buf, sizeof(buf), fmt, a...); out += buf; };
    out += "ann\n";
    put("ntypes %i\n", ntypes());
    for (auto& x : sp) {  // Type::write (type.cpp:148-164)
        put("name %s ", x.name.c_str());
        if (x.has_mass) put("mass %f ", x.mass);
        if (x.has_energy) put("energy %f ", x.energy);
        out += "\n";
    }
    put("rc %f\n", rc);
    for (int i = 0; i < ntypes(); ++i) {
        put("basis %s\n", sp[i].name.c_str());
        for (int j = 0; j < ntypes(); ++j) {
            put("basis_radial %s\n", sp[j].name.c_str());
            const BasisR& b = sp[i].R[j];
            put("BasisR %s %f %s %i\n", cut_name(b.cut.name), b.cut.rc, radial_name(b.name), b.size());
            for (int m = 0; m < b.size(); ++m) put("\t%f %f\n", b.rs[m], b.eta[m]);
        }
        for (int j = 0; j < ntypes(); ++j) for (int k = j; k < ntypes(); ++k) {
            put("basis_angular %s %s\n", sp[j].name.c_str(), sp[k].name.c_str());
            const BasisA& b = sp[i].A[tri_index(j, k)];
            put("BasisA %s %f %s %i\n", cut_name(b.cut.name), b.cut.rc, angular_name(b.name), b.size());
            for (int m = 0; m < b.size(); ++m) put("\t%f %f %i %i\n", b.eta[m], b.zeta[m], b.lambda[m], b.rflag[m]);
        }
    }
    for (auto& x : sp) {  // ANN::write (nn.cpp:1436-1474)
        put("nn %s\n", x.name.c_str());
        const Network& nn = x.nn;
        put("nn %i ", nn.nin);
        for (int l = 0; l < nn.nlayer(); ++l) put("%i ", nn.nodes[l]);
        out += "\n";
        put("neuron %s %f\n", neuron_names[nn.neuron], nn.c);
        out += "inpw "; for (double v : nn.inpw) put("%.15f ", v); out += "\n";
        out += "outw "; for (double v : nn.outw) put("%.15f ", v); out += "\n";
        out += "inpb "; for (double v : nn.inpb) put("%.15f ", v); out += "\n";
        out += "outb "; for (double v : nn.outb) put("%.15f ", v); out += "\n";
        for (int l = 0; l < nn.nlayer(); ++l) { put("bias[%i] ", l + 1); for (double v : nn.b[l]) put("%.15f ", v); out += "\n"; }
        for (int l = 0; l < nn.nlayer(); ++l) { put("weight[%i,%i] ", l, l + 1); for (double v : nn.w[l]) put("%.15f ", v); out += "\n"; }
    }
    return out;
}

void Potential::validate() const {
    for (auto& x : sp) {
        if (x.nn.nodes.back() != 1) throw ann_error(ANN_ERR_UNSUPPORTED, "networks must have one output (type " + x.name + ")");
        const int act = x.nn.neuron;
        if (act <= N_UNKNOWN || act > N_TEST)
            throw ann_error(ANN_ERR_UNSUPPORTED, "activation " + std::to_string(act) + " is not implemented on the GPU path");
        for (int l = 0; l < x.nn.nlayer(); ++l)
            if (x.nn.nodes[l] > 256) throw ann_error(ANN_ERR_UNSUPPORTED, "layers wider than 256 nodes are not supported");
        if (x.nInput > 256) throw ann_error(ANN_ERR_UNSUPPORTED, "more than 256 inputs per atom are not supported");
        // all basis blocks of one centre type share one cutoff (evaluated once per neighbour)
        const Cutoff* c0 = nullptr;
        for (auto& b : x.R) { if (b.size() == 0) continue; if (!c0) c0 = &b.cut; else if (b.cut.name != c0->name || b.cut.rc != c0->rc) throw ann_error(ANN_ERR_UNSUPPORTED, "basis blocks of one type must share a cutoff"); }
        for (auto& b : x.A) { if (b.size() == 0) continue; if (!c0) c0 = &b.cut; else if (b.cut.name != c0->name || b.cut.rc != c0->rc) throw ann_error(ANN_ERR_UNSUPPORTED, "basis blocks of one type must share a cutoff"); }
        if (c0 && c0->rc > rc) throw ann_error(ANN_ERR_UNSUPPORTED, "basis cutoff larger than the potential cutoff");
        for (auto& b : x.R) if (b.size() > 64) throw ann_error(ANN_ERR_UNSUPPORTED, "more than 64 radial functions per block");
        for (auto& b : x.A) if (b.size() > 64) throw ann_error(ANN_ERR_UNSUPPORTED, "more than 64 angular functions per block");
    }
    if (ntypes() > 8) throw ann_error(ANN_ERR_UNSUPPORTED, "more than 8 types");
}

// ------------------------------------------------------------------ ANN::resize initialisation
void init_network(Network& nn, int seed, int dist, int init, double sigma_b, double sigma_w) {
    if (sigma_b <= 0) throw ann_error(ANN_ERR_ARG, "invalid initialization deviation - bias");    // nn.cpp:1074
    if (sigma_w <= 0) throw ann_error(ANN_ERR_ARG, "invalid initialization deviation - weight");  // nn.cpp:1075
    std::mt19937 rngen(seed);
    auto factor = [&](int n) {
        const int ni = nn.ni(n), no = nn.nodes[n];
        switch (init) {
            case 1: return 1.0;                                  // RAND
            case 2: return std::sqrt(1.0 / ni);                  // LECUN
            case 3: return std::sqrt(2.0 / ni);                  // HE
            case 4: return std::sqrt(2.0 / (no + ni));           // XAVIER
            default: throw ann_error(ANN_ERR_ARG, "invalid initialization scheme");
        }
    };
    const int L = nn.nlayer();
    nn.b.assign(L, {}); nn.w.assign(L, {});
    for (int n = 0; n < L; ++n) { nn.b[n].assign(nn.nodes[n], 0.0); nn.w[n].assign(nn.nodes[n] * nn.ni(n), 0.0); }
    // biases (nn.cpp:1123-1139), a fresh distribution object per layer
    for (int n = 0; n < L; ++n) {
        if (dist == 1) {
            const double s = std::sqrt(3.0 * sigma_b) * factor(n);
            std::uniform_real_distribution<double> d(-s, s);
            for (auto& v : nn.b[n]) v = d(rngen);
        } else {
            std::normal_distribution<double> d(0.0, sigma_b * factor(n));
            for (auto& v : nn.b[n]) v = d(rngen);
        }
    }
    // weights (nn.cpp:1140-1190): Eigen storage is column-major, element k -> (row k%rows, col k/rows)
    for (int n = 0; n < L; ++n) {
        const int rows = nn.nodes[n], cols = nn.ni(n);
        if (dist == 1) {
            const double s = std::sqrt(3.0 * sigma_w) * factor(n);
            std::uniform_real_distribution<double> d(-s, s);
            for (int k = 0; k < rows * cols; ++k) nn.w[n][(k % rows) * cols + k / rows] = d(rngen);
        } else {
            std::normal_distribution<double> d(0.0, sigma_w * factor(n));
            for (int k = 0; k < rows * cols; ++k) nn.w[n][(k % rows) * cols + k / rows] = d(rngen);
        }
    }
}

}  // namespace ann
