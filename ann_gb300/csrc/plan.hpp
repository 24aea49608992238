// Flattened, device-visible description of a loaded potential (passed by value as a
// __grid_constant__ kernel parameter) plus the per-batch kernel argument blocks.
// Shared by host (plan.cpp, context.cu) and device code.
#pragma once
#include <cstdint>

namespace ann {

// 4-vectors of one neighbour entry (rx, ry, rz, d); explicit alignment so that the bulk
// copies and vector loads of neighbour rows are always aligned
struct alignas(16) Vec4f { float x, y, z, w; };
struct alignas(32) Vec4d { double x, y, z, w; };

constexpr int MAXT = 4;                          // types per potential
constexpr int MAXBLK = MAXT * (MAXT + 1) / 2;    // angular blocks per centre type
constexpr int NGMAX = 4;                         // damping groups (distinct eta) per centre type
constexpr int MAXLAYER = 6;                      // weight layers per network
constexpr int MAXW = 256;                        // widest layer / input vector

// status word bits (device int status[0])
enum StatusBits {
    ST_NBR_OVERFLOW = 1,    // an atom had more neighbour entries than the list capacity
    ST_IMAGE_RANGE = 2,     // an atom is more than 500 cells away from the home cell
    ST_BAD_TYPE = 4,        // type index out of range
    ST_TIMEOUT = 8,         // a bounded mbarrier wait gave up
    ST_NONFINITE = 16,      // non-finite position
    ST_BAD_INDEX = 32,      // a caller's neighbour list names an atom outside [0, nall)
};

struct DevRadial {          // BasisR block (I,J)
    int32_t name, n, off, pidx;        // off: input offset; pidx: first parameter in rs[]/eta[]
};
struct DevAngular {         // BasisA block (I,JK)
    int32_t name, n, off, pidx;        // pidx: first parameter in aeta[]/zeta[]/lam[]/agrp[]
    int32_t sidx;                      // first entry of slot2ref[] (fast path), -1 if not fast
};
struct DevNet {
    int32_t nlayer, nin, neuron;
    int32_t nodes[MAXLAYER];
    int32_t woff[MAXLAYER], boff[MAXLAYER];   // offsets into the weight / bias arrays
    int32_t inoff;                            // offset of inpw / inpb in the input-scaling arrays
    double c, outw, outb;
};
struct DevType {
    int32_t nInput, nInputR;
    int32_t cut;                       // cutoff name shared by the type's blocks (CUT_*)
    int32_t ngroups;                   // distinct angular eta of the type (fast path)
    double rc;                         // basis cutoff radius
    double ietar2[NGMAX];              // 1/eta_g^2 per damping group
    double evac;                       // per-type vacuum energy (Type::energy)
    DevRadial R[MAXT];
    DevAngular A[MAXBLK];
    DevNet net;
};
struct DevPot {
    int32_t ntypes, imax;
    int32_t fast;                      // 1: every angular block is GAUSS with lambda=+-1, zeta=2^k (k<=3)
    int32_t fastNG;                    // damping groups compiled into the fast kernels (1,2,4)
    double rc;                         // neighbour cutoff (NNP::rc)
    int32_t nrad, nslot;               // lengths of the radial parameter arrays (rs / reta) and of slot2ref
    DevType t[MAXT];
};

// device pointers of the potential's parameter arrays, per precision
template <typename real>
struct DevParams {
    const real* rs;        // radial rs
    const real* reta;      // radial eta
    const real* aeta;      // angular eta
    const real* zeta;      // angular zeta
    const real* alam;      // angular lambda (as real)
    const int32_t* agrp;   // angular: damping group index (into the type's ietar2)
    const int32_t* slot2ref;  // fast path: slot -> index within block (or -1)
    const real* w;         // network weights, row-major per layer (rows = outputs)
    const real* wt;        // transposed copies (rows = inputs)
    const real* b;         // biases
    const real* inpw;      // input scaling
    const real* inpb;
};

}  // namespace ann
