/*
 * ann_gpu.h -- C ABI of the GB300 Behler-Parrinello energy/force library (libann_gpu.so).
 *
 * Drop-in boundary for the compute call of markdellostritto/ann ("AtomicNN"): it replaces
 *   NNP::read / NNP::write                     src/nnp/nnp.cpp:181-307 (+ ANN text IO src/ml/nn.cpp:1436-1578)
 *   NNP::init + NNP::symm + NNP::energy        src/nnp/nnp.cpp:316-447
 *   NNP::force / NNP::compute                  src/nnp/nnp.cpp:461-736
 *   ptnl::PotNNPE::compute (energy incl. E_vac) src/torch/pot_nnpe.cpp:169-288
 *   NeighborList(struc, rc) build               src/struc/ (missing; contract from src/nnp/nnp.cpp:343-348)
 *   ANN::operator>> / operator<< param packing src/ml/nn.cpp:846-880
 *   NNPTEFR::error_cost_o1 energy gradient      src/nnp/nnptefr2.cpp:1321-1374, 984-995
 *   NNPTE::error force-term gradient            src/nnp/nnptef.cpp:1560-1936
 *   Verlet::compute MD step                      src/torch/integrator.cpp:177-200
 *
 * Conventions (metal units: eV, Angstrom, fs, Dalton):
 *  - every function returns 0 (ANN_OK) or an ANN_ERR_* code; ann_last_error() gives the text.
 *    No C++ exception crosses this boundary (the reference throws std::invalid_argument /
 *    std::runtime_error for the same conditions).
 *  - the caller owns all host arrays; the context owns its device buffers, one CUDA stream and
 *    captured CUDA graphs. A context is not reentrant (like the reference's NNP, which keeps
 *    per-call scratch): use one context per host thread.
 *  - a batch is nstruc structures packed back to back: atom_offsets[nstruc+1] (atom_offsets[0]=0),
 *    posn[3*N] (x,y,z per atom), type[N] (index into the potential's types, see
 *    ann_type_index), cell[9*nstruc] (per structure the 3x3 lattice matrix R column-major:
 *    cell[9*s + 3*c + r] = R[r][c], lattice vectors are the columns, as Structure::R()).
 *  - neighbours: every periodic image j + R n with |x_i - x_j - R n| < rc, except j==i, n==0.
 *  - forces: F = -dE/dx (3N); energies per structure include the per-type vacuum energies
 *    (NNH::energy src/nnp/nnh.cpp:118-121). virial per structure W[a*3+b] = sum over centre atoms
 *    i and neighbours j of r_ij[a] * v_ij[b], v_ij = -dE_i/dr_ij (so dE/d(strain)_ab = -W_ba).
 */
#ifndef ANN_GPU_H
#define ANN_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ANN_GPU_ABI_VERSION 4

enum ann_status {
    ANN_OK = 0,
    ANN_ERR_ARG = 1,          /* invalid argument (null pointer, bad size, bad type index)          */
    ANN_ERR_IO = 2,           /* file could not be opened / written                                  */
    ANN_ERR_FORMAT = 3,       /* malformed potential file                                            */
    ANN_ERR_CUDA = 4,         /* CUDA runtime error (no device, launch failure, out of memory)       */
    ANN_ERR_CAPACITY = 5,     /* a device capacity was exceeded and could not be grown               */
    ANN_ERR_STATE = 6,        /* call out of order (no potential loaded, no batch, no forward pass)  */
    ANN_ERR_TIMEOUT = 7,      /* a bounded device-side wait gave up                                  */
    ANN_ERR_UNSUPPORTED = 8,  /* valid input the GPU path does not implement (named in the message)  */
    ANN_ERR_NUMERIC = 9       /* non-finite positions / cell, or non-finite results                  */
};

enum ann_precision {
    ANN_FP64 = 0,   /* plain form: FP64 geometry, basis, network and forces                          */
    ANN_MIXED = 1   /* FP32 geometry/basis/forces, FP32-accumulated network, FP64 energy sums       */
};

enum ann_newton {
    ANN_NEWTON_ALL_IMAGES = 0,    /* Newton-3rd force on every neighbour entry (exact -dE/dx)        */
    ANN_NEWTON_UNTRANSLATED = 1   /* only for image n==0: the verlet::List rule of nnp.cpp:550       */
};

typedef struct ann_options {
    int32_t device;              /* CUDA device ordinal                                               */
    int32_t precision;           /* default precision for calls that do not name one (ann_precision)  */
    int32_t newton;              /* ann_newton                                                         */
    int32_t max_neighbors;       /* initial neighbour capacity per atom (0 = estimate from density)   */
    int32_t use_graphs;          /* capture the per-batch kernel sequence in a CUDA graph (1 = yes)   */
    int32_t mlp_backend;         /* 0 = auto, 1 = SIMT kernels, 2 = tcgen05 tensor-core kernels (MIXED) */
    int32_t tc_groups;           /* tensor-core network kernel: warps per TMEM lane quadrant, 1, 2 or 4 */
                                 /* (4 / tc_groups CTAs per SM); 0 = chosen per launch                 */
    int32_t tc_split;            /* tensor-core network operands: 1 = single BF16 activations and       */
                                 /* weights, 2 = activations split hi + lo (2 MMAs per k-step), 3 = both */
                                 /* split (3 MMAs); 0 = the most accurate form whose image fits shared  */
                                 /* memory. A type whose networks fit no allowed form runs on SIMT      */
} ann_options;

typedef struct ann_ctx ann_ctx;

/* ---- lifetime ------------------------------------------------------------------------------ */
void ann_default_options(ann_options* opt);
int ann_create(ann_ctx** ctx, const ann_options* opt);   /* opt may be NULL (defaults)             */
int ann_destroy(ann_ctx* ctx);
const char* ann_last_error(const ann_ctx* ctx);          /* ctx may be NULL: last global error      */
int ann_abi_version(void);

/* ---- potential: NNP::read / NNP::write (nnp.cpp:181-307), params (nn.cpp:846-880) ----------- */
int ann_load_potential(ann_ctx* ctx, const char* path);
int ann_load_potential_text(ann_ctx* ctx, const char* text);
int ann_write_potential(ann_ctx* ctx, const char* path);
int ann_num_types(ann_ctx* ctx, int32_t* ntypes);
int ann_type_index(ann_ctx* ctx, const char* name, int32_t* index);   /* NNP::index (nnp.hpp)      */
int ann_type_name(ann_ctx* ctx, int32_t index, char* buf, int32_t buflen);
int ann_cutoff(ann_ctx* ctx, double* rc);
int ann_num_inputs(ann_ctx* ctx, int32_t type, int32_t* ninput);       /* NNH::nInput               */
/* The form the MIXED network pass takes for a type (no reference counterpart): backend 2 = tcgen05
 * tensor cores with split = 1, 2 or 3 (ann_options.tc_split), 1 = SIMT kernel (split 0).          */
int ann_network_form(ann_ctx* ctx, int32_t type, int32_t* backend, int32_t* split);
int ann_num_params(ann_ctx* ctx, int64_t* nparams);                     /* NNP::size (nnp.cpp:47-53) */
int ann_get_params(ann_ctx* ctx, double* params, int64_t nparams);      /* types in NNP order        */
int ann_set_params(ann_ctx* ctx, const double* params, int64_t nparams);
/* input pre-conditioning ins = inpw*(G+inpb) of one type's network (nn.cpp:1343-1346)            */
int ann_set_input_scaling(ann_ctx* ctx, int32_t type, const double* inpw, const double* inpb, int32_t ninput);
/* Xavier/He/LeCun/random initialisation of one type's network exactly as ANN::resize
 * (nn.cpp:1071-1190: std::mt19937(seed), biases then weights, column-major; dist 0 = NORMAL,
 * 1 = UNIFORM; init 1 RAND, 2 LECUN, 3 HE, 4 XAVIER)                                              */
int ann_init_network(ann_ctx* ctx, int32_t type, int32_t seed, int32_t dist, int32_t init,
                     double sigma_b, double sigma_w);

/* ---- compute: nnpce loop / NNP::compute / PotNNPE::compute over a batch (host buffers) ------ */
int ann_compute(ann_ctx* ctx, int32_t nstruc, const int64_t* atom_offsets, const double* posn,
                const int32_t* type, const double* cell, double* energy /* nstruc */,
                double* forces /* 3N or NULL */, double* virial /* 9*nstruc or NULL */,
                int32_t precision);

/* ---- compute from the caller's neighbour list: an MD engine's domain with ghost atoms ---------
 * The shape of LAMMPS `pair_style nn <rc>` / `pair_coeff * * <ann file> <elements>` (the
 * reference runs it at examples/Ar/Ar_md_npt.in:22-23; that pair style's source is not part of
 * the reference) and of NNP::compute(nnp, struc, nlist) (src/nnp/nnp.cpp:601-665), where the
 * caller owns the neighbour list.
 *  - nall atoms (local then ghost, as LAMMPS orders them): x[3*nall] positions, ghosts already
 *    shifted to their image; type[nall] potential type indices (ann_type_index).
 *  - inum rows, one per centre atom: ilist[inum] the centre atom of each row (NULL: row r is
 *    atom r); numneigh[inum] the row lengths; neigh[] the rows back to back, atom indices in
 *    [0, nall) (LAMMPS: firstneigh[i][k] & NEIGHMASK). The list must be FULL (every neighbour of
 *    every centre). Entries at or beyond the potential's cutoff are ignored, so a list built with
 *    a skin may be passed as it is.
 *  - energy[1]: sum over the rows of the atomic energies (incl. vacuum energies); eatom[inum]
 *    (or NULL): the energy of each row's atom, in row order.
 *  - forces[3*nall] (or NULL) is overwritten with -dE/dx of every local AND ghost atom; with
 *    newton_pair on the engine adds the ghost forces to their owners (LAMMPS reverse_comm).
 *  - virial[9] (or NULL): sum over rows and entries of r[a] * v[b] as for ann_compute (LAMMPS
 *    virial[0..5] = W[0], W[4], W[8], W[1], W[2], W[5]).
 *  - flags: 0, or ANN_LIST_KEEP when the list, ilist, types and nall are those of the previous
 *    call on this context and only x changed (an MD engine between two reneighbourings; LAMMPS:
 *    neighbor->ago != 0). ilist, numneigh, neigh and type may then be NULL; only x is copied to
 *    the device. The cutoff filter still runs on the new positions, so a list with a skin stays
 *    exact while atoms move within it.
 * Index, type or non-finite position errors return ANN_ERR_ARG / ANN_ERR_NUMERIC.                 */
#define ANN_LIST_KEEP 1
int ann_compute_list(ann_ctx* ctx, int32_t inum, const int32_t* ilist, const int32_t* numneigh,
                     const int32_t* neigh, int32_t nall, const double* x, const int32_t* type,
                     double* energy, double* eatom /* inum or NULL */, double* forces /* 3*nall or NULL */,
                     double* virial /* 9 or NULL */, int32_t precision, int32_t flags);

/* ---- compute with device-resident batches -------------------------------------------------- */
/* Stage a batch (host pointers; copied to the context's device buffers).                        */
int ann_batch_upload(ann_ctx* ctx, int32_t nstruc, const int64_t* atom_offsets, const double* posn,
                     const int32_t* type, const double* cell);
/* Stage a batch from device pointers already on the context's device (copied device-to-device
 * on the context stream; atom_offsets is a HOST array here, posn/type/cell are device pointers).  */
int ann_batch_set_device(ann_ctx* ctx, int32_t nstruc, const int64_t* atom_offsets,
                         const double* d_posn, const int32_t* d_type, const double* d_cell);
/* Run the E+F pipeline on the staged batch; asynchronous on the context stream.                  */
int ann_batch_compute(ann_ctx* ctx, int32_t precision, int32_t want_forces);
/* Wait for the batch and copy results to host buffers (NULL = skip); grows capacities and
 * recomputes transparently if a neighbour list overflowed.                                       */
int ann_batch_download(ann_ctx* ctx, double* energy, double* forces, double* virial);
/* Same results into device pointers (double) on the context's device; synchronises.              */
int ann_batch_results_device(ann_ctx* ctx, double* d_energy, double* d_forces, double* d_virial);
int ann_synchronize(ann_ctx* ctx);
/* Page-locked host memory on the context's device (cudaMallocHost): inputs built there and
 * results read into it are copied by DMA without staging, asynchronously on the context stream.
 * For callers that feed many batches (a data loader, an MD engine's arrays). Free with
 * ann_host_free (ctx may be NULL there: a buffer may outlive its context); bytes = 0 returns
 * NULL.                                                                                           */
int ann_host_alloc(ann_ctx* ctx, int64_t bytes, void** ptr);
int ann_host_free(ann_ctx* ctx, void* ptr);
/* Raw CUDA stream of the context (cudaStream_t), for callers timing or ordering around it.      */
void* ann_stream(ann_ctx* ctx);

/* ---- instrumentation (no counterpart in the reference, which prints wall-clock phase timers,
 *      nnptefr2.cpp:3374-3400) ------------------------------------------------------------------- */
/* Total kernels this context has launched (graph replays count their kernel nodes).             */
int ann_kernel_count(ann_ctx* ctx, int64_t* launches);
/* enable = 1: subsequent batches run without graph capture and record CUDA events around each
 * phase on the context stream; ann_phase_times returns the last batch's phase durations in ms:
 * [0] neighbour list, [1] type lists, [2] symmetry functions, [3] networks, [4] forces,
 * [5] per-structure reductions.                                                                  */
int ann_profile_phases(ann_ctx* ctx, int32_t enable);
int ann_phase_times(ann_ctx* ctx, double* ms, int32_t n);

/* ---- inspection (parity tests) -------------------------------------------------------------- */
/* Max inputs over types: rows of ann_get_symm / ann_get_dedg are padded to this width.           */
int ann_symm_width(ann_ctx* ctx, int32_t* width);
/* The output capacities (in doubles) are checked against the last batch: N*width, N*width, N.  */
int ann_get_symm(ann_ctx* ctx, double* symm, int64_t cap);        /* NNP::symm of last batch     */
int ann_get_dedg(ann_ctx* ctx, double* dedg, int64_t cap);        /* dE_i/dG_i (DODZ::dodi row 0) */
int ann_get_atom_energies(ann_ctx* ctx, double* e, int64_t cap);
/* neighbour list of the last batch: total entries, then (i, j, image n0,n1,n2) per entry.        */
int ann_num_neighbors(ann_ctx* ctx, int64_t* total);
int ann_get_neighbors(ann_ctx* ctx, int32_t* i_out, int32_t* j_out, int32_t* img_out /* 3 per */,
                      double* r_out /* 3 per, FP64 pipelines only else NULL */, int64_t cap);

/* ---- training: forward/backward pair (the contract of a torch.autograd.Function) ------------ */
/* L = wE/S sum_s 1/2 ((E_s-Eref_s)/N_s)^2 + wF/(3N) sum_a 1/2 |F_a-Fref_a|^2 (energy term: see ann_train_set_loss)
 * (energy term = NNPTEFR::error_cost_o1 MSE/LINEAR, nnptefr2.cpp:1321-1374 + 984-995;
 *  force term = the intent of NNPTE::error, nnptef.cpp:1715-1825, with all neighbour terms).
 * loss3 = {L, L_E, L_F}. Saves the state the backward pass needs on the device.                 */
int ann_train_forward(ann_ctx* ctx, int32_t nstruc, const int64_t* atom_offsets, const double* posn,
                      const int32_t* type, const double* cell, const double* energy_ref,
                      const double* forces_ref, double w_energy, double w_force, int32_t precision,
                      double* loss3);
/* The same forward pass over the structures and labels of the preceding ann_train_forward, whose
 * neighbour rows, per-type atom lists and symmetry functions stay on the device: the reference
 * trainer builds each structure's neighbour list and symmetry functions once, before optimising
 * (nnptefr2.cpp:2690-2703), and every step evaluates the networks on the stored symm
 * (error_cost_o1, nnptefr2.cpp:1321-1374). Each call runs the networks, the forces, the
 * per-structure sums and the loss with the current parameters (after optimiser steps,
 * ann_set_params or new input scaling). ANN_ERR_STATE if no ann_train_forward preceded it, if
 * another batch, E+F call, MD step or potential load came in between, or if precision differs
 * from that call's. ann_train_backward follows it as it follows ann_train_forward.             */
int ann_train_forward_staged(ann_ctx* ctx, double w_energy, double w_force, int32_t precision, double* loss3);
/* The energy term's loss and normalisation for later ann_train_forward calls (NNPTEFR,
 * nnptefr2.cpp:1339-1368, normalisation 606-612). For structure s with dU = (E_s - Eref_s) normt(N_s):
 * MSE 1/2 dU^2, MAE |dU|, HUBER delta^2 (sqrt(1 + (dU/delta)^2) - 1), ASINH delta^2 (1 - sqrt(1 + a^2)
 * + a asinh(a)) with a = dU/delta; normt = 1, 1/N, 1/sqrt(N), 1/cbrt(N), 1/(ln N + 1). The
 * energy term of L is wE/S sum_s loss_s. The default is MSE with LINEAR. The force term stays the
 * mean squared error. Enum values are those of opt::Loss (opt/loss.hpp:18-24) and Norm
 * (nnptefr2.hpp:119-126).                                                                         */
enum ann_loss { ANN_LOSS_MSE = 1, ANN_LOSS_MAE = 2, ANN_LOSS_HUBER = 3, ANN_LOSS_ASINH = 4 };
enum ann_norm { ANN_NORM_IDENTITY = 0, ANN_NORM_LINEAR = 1, ANN_NORM_SQRT = 2, ANN_NORM_CBRT = 3, ANN_NORM_LOG = 4 };
int ann_train_set_loss(ann_ctx* ctx, int32_t loss, int32_t norm, double delta);
/* dL/dp (reference packing, types in NNP order) scaled by dl_scale. Requires ann_train_forward.
 * grad may be NULL: the gradient then stays on the device only, for ann_adam_step.               */
int ann_train_backward(ann_ctx* ctx, double dl_scale, double* grad, int64_t nparams);
/* Adam optimiser on the device (NN::ADAM::step, opt/algo.cpp:272-296): ann_adam_init sets the
 * step size (gamma), beta1, beta2, eps and zeroes the moments; each ann_adam_step applies one
 * step with the gradient of the preceding ann_train_backward times scale, to the parameters held
 * on the device (FP64 master and every FP32 / tensor-core copy), so that a training loop needs no
 * parameter transfer. ann_get_params / ann_write_potential read the updated parameters.       */
int ann_adam_init(ann_ctx* ctx, double lr, double beta1, double beta2, double eps);
int ann_adam_step(ann_ctx* ctx, double scale);
/* The trainer's step-size schedule and weight decay around every optimiser step (nnptefr2.cpp:1025-1049):
 * before step t (counted from 0 since the optimiser's init), gamma <- decay(gamma, t) with DECAY / ALPHA /
 * PERIOD as opt::Decay (opt/decay.cpp:42-62): CONST gamma, EXP gamma (1 - alpha), GAUSS
 * gamma (1 - 2 alpha t), SQRT gamma (1 - alpha / (2 (1 + alpha t))), INV gamma (1 - alpha /
 * (1 + alpha t)), STEP gamma alpha every PERIOD steps. After the step, the weights (not the biases)
 * get p -= gamma eta f(p_old), with f = sgn (LASSO), x (RIDGE), x / sqrt(1 + x^2) (HUBER), or asinh
 * (ASINH); REG_NONE skips this. The default is CONST and NONE. Enum values are those of opt::Decay
 * (opt/decay.hpp:28-36) and Regularization (nnptefr2.hpp:173-181).                               */
enum ann_decay { ANN_DECAY_CONST = 1, ANN_DECAY_EXP = 2, ANN_DECAY_GAUSS = 3, ANN_DECAY_SQRT = 4, ANN_DECAY_INV = 5, ANN_DECAY_STEP = 6 };
enum ann_reg { ANN_REG_LASSO = 0, ANN_REG_RIDGE = 1, ANN_REG_HUBER = 2, ANN_REG_ASINH = 3, ANN_REG_NONE = 4 };
int ann_opt_set_schedule(ann_ctx* ctx, int32_t decay, double alpha, int32_t period, int32_t reg, double eta);
/* Any optimiser of the reference trainer (opt::algo, src/opt/algo.cpp:97-660) on the device, with
 * the values of opt::algo::Name (src/opt/algo.hpp:31-49). gamma is the step size, eta the momentum
 * / decay of SDM, NAG and ADADELTA, eps the denominator's guard, and w ADAMW's weight decay. The
 * Adam family uses beta1 = 0.9, beta2 = 0.999 as the reference; ann_adam_init takes other betas.
 * RPROP compares the loss of the last ann_train_forward with the loss at the previous step. BFGS
 * keeps a dense P x P matrix and returns ANN_ERR_UNSUPPORTED. ann_opt_step applies one step with
 * the gradient of the preceding ann_train_backward (times scale), like ann_adam_step.            */
enum ann_opt {
    ANN_OPT_SGD = 1, ANN_OPT_SDM = 2, ANN_OPT_NAG = 3, ANN_OPT_ADAGRAD = 4, ANN_OPT_ADADELTA = 5, ANN_OPT_RMSPROP = 6,
    ANN_OPT_ADAM = 7, ANN_OPT_ADAMW = 8, ANN_OPT_ADAB = 9, ANN_OPT_YOGI = 10, ANN_OPT_NOGI = 11, ANN_OPT_NADAM = 12,
    ANN_OPT_AMSGRAD = 13, ANN_OPT_BFGS = 14, ANN_OPT_RPROP = 15, ANN_OPT_CG = 16
};
int ann_opt_init(ann_ctx* ctx, int32_t algo, double gamma, double eta, double eps, double w);
int ann_opt_step(ann_ctx* ctx, double scale);

/* ---- input statistics and pre-conditioning of a training set (nnptefr2.cpp:686-858) ----------
 * The trainer's set-up: statistics of every input over all atoms of each type in the training
 * set, then inpb / inpw of each network from them. Accumulated on the device batch by batch:
 * ann_stats_accumulate adds the symmetry functions of the last computed batch (ann_compute,
 * ann_batch_compute or ann_train_forward; in that call's precision, FP64 to match the reference).
 * ann_stats_get gives, for type t, count = atoms accumulated and stats[6 * nInput(t)] = rows max,
 * min, harmonic mean N/sum(1/G), mean, standard deviation (N-1 normalised; 0 for N < 2) and rms.
 * ann_precondition sets, for every type with atoms, inpb = bias(prebias) + inbias and
 * inpw = scale(prescale) * inscale, and outb = 0, outw = 1, as the trainer does. Enum values are
 * those of PreBias / PreScale (nnptefr2.hpp:59-97).                                              */
enum ann_prebias {
    ANN_PREBIAS_IDENTITY = 0, ANN_PREBIAS_MEAN = 1, ANN_PREBIAS_HAR = 2, ANN_PREBIAS_RMS = 3, ANN_PREBIAS_MID = 4,
    ANN_PREBIAS_MIN = 5
};
enum ann_prescale { ANN_PRESCALE_IDENTITY = 0, ANN_PRESCALE_DEV = 1, ANN_PRESCALE_MINMAX = 2, ANN_PRESCALE_MAX = 3 };
int ann_stats_reset(ann_ctx* ctx);
int ann_stats_accumulate(ann_ctx* ctx);
int ann_stats_get(ann_ctx* ctx, int32_t type, int64_t* count, double* stats);
int ann_precondition(ann_ctx* ctx, int32_t prebias, int32_t prescale, double inbias, double inscale);
/* the input scaling of type t's network (inpw, inpb; n = nInput(t))                               */
int ann_get_input_scaling(ann_ctx* ctx, int32_t type, double* w, double* b, int32_t n);

/* ---- molecular dynamics: velocity Verlet (integrator.cpp:177-200) --------------------------- */
/* One structure; masses per type in Dalton. list_skin adds to rc for the Verlet list; the list is
 * rebuilt when an atom has moved more than skin/2 since the last build.                          */
int ann_md_init(ann_ctx* ctx, int64_t natoms, const double* posn, const double* vel,
                const int32_t* type, const double* cell, const double* mass_per_type,
                double dt_fs, double list_skin, int32_t precision);
/* nsteps velocity-Verlet steps, captured as one CUDA graph per step. pe/ke (eV) after the last
 * step; rebuilds = number of neighbour-list rebuilds during the call.                            */
int ann_md_run(ann_ctx* ctx, int32_t nsteps, double* pe, double* ke, int32_t* rebuilds);
int ann_md_get_state(ann_ctx* ctx, double* posn, double* vel, double* forces);

/* ---- network pass without device allocation (no counterpart in the reference) ---------------
 * The network stage of ann_compute alone: energy per atom (network output + vacuum energy) and
 * dE/dG for symmetry functions that are already on the device. All pointers are device memory:
 * type_dev[natoms] (int32), G_dev and dEdG_dev [natoms * ann_symm_width] (double for ANN_FP64,
 * float for ANN_MIXED), Eatom_dev[natoms] (double). Runs on ann_stream(ctx); returns after the
 * stream has finished and the device status has been checked.
 * It allocates no device memory, for callers that must not allocate during a step (an MD engine
 * or plugin host that reserves its device memory up front; cudaMalloc/cudaFree synchronise the
 * device and can fail mid-run). Its scratch is one static device array of the library,
 * ANN_NOALLOC_SCRATCH_BYTES, shared by every call on a device: calls that overlap in time
 * (other threads, contexts or streams) race on it and must be serialised by the caller.
 * natoms > ANN_NOALLOC_MAX_ATOMS returns ANN_ERR_CAPACITY; natoms = 0 does nothing. Every call
 * looks the array's device address up (cudaGetSymbolAddress, a host query that allocates nothing).
 * The call is synchronous: it ends with a copy of the status word to host memory and a stream
 * synchronisation, so it must not be called while ann_stream(ctx), or the legacy default stream,
 * is being captured into a CUDA graph.                                                          */
#define ANN_NOALLOC_MAX_ATOMS 262144
#define ANN_NOALLOC_SCRATCH_BYTES (2 * 1024 * 1024 + 4096)
int ann_network_noalloc(ann_ctx* ctx, int32_t natoms, const int32_t* type_dev, const void* G_dev,
                        double* Eatom_dev, void* dEdG_dev, int32_t precision);

/* ---- launch-shape autotuner --------------------------------------------------------------------
 * The run-time launch shapes of the E+F sequence are timed on the staged batch (the structures of
 * the last ann_compute call), each through its own captured CUDA graph:
 *   - per type, the warps per TMEM lane quadrant of the tensor-core network kernel: 1, 2 or 4,
 *     giving 4, 2 or 1 CTAs per SM (MIXED on the tensor-core kernel only);
 *   - the resident blocks per SM of the symmetry-function and force passes;
 *   - the blocks per SM of the neighbour search.
 * The search is coordinate-wise: each knob over its candidates with the others held, keeping a
 * candidate only when it beats the best so far by more than 1 %. Each candidate takes the median
 * of `reps` timed evaluations (CUDA events).
 * The context keeps the choice for its later calls. A 0 field is the built-in rule; for
 * tc_groups that is ann_options.tc_groups, itself 0 for the per-launch rule. A failed search
 * leaves the shapes the context had before it.
 * ann_set_tuning applies a stored choice. The staged batch is recomputed, with the same results.
 * Not in MD mode (ANN_ERR_STATE). */
typedef struct ann_tuning {
    int32_t tc_groups[4];          /* per type: 1, 2, 4, or 0 for the per-launch rule               */
    int32_t bp_blocks_per_sm;      /* symmetry / force passes: 1..16, or 0 for as many as fit       */
    int32_t nbr_blocks_per_sm;     /* neighbour search: 1..64, or 0 for 16                           */
    double ms;                     /* ann_autotune: one evaluation with the chosen shapes (ms)       */
    double ms_default;             /* ann_autotune: one evaluation with every field 0 (ms)           */
} ann_tuning;
int ann_autotune(ann_ctx* ctx, int32_t precision, int32_t reps, ann_tuning* out);

/* ---- bounded device waits (testing aid; no counterpart in the reference) -----------------------
 * Every device-side wait (a staged neighbour row, a network weight image, a tensor-core MMA) gives
 * up after a bounded number of polls, reports ANN_ERR_TIMEOUT, lets its copies and MMAs finish
 * (with the full bound) and returns, so the context stays usable. polls >= 0 makes those waits
 * give up after that many non-blocking polls (0: at once, every time), which exercises the
 * timeout path without a fault or a hang; -1 (the default) restores the built-in bounds. The
 * launch graphs are recaptured on the next call.                                                  */
int ann_set_wait_limit(ann_ctx* ctx, int32_t polls);
int ann_set_tuning(ann_ctx* ctx, const ann_tuning* t);

#ifdef __cplusplus
}
#endif
#endif /* ANN_GPU_H */
