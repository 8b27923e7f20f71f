// Scheme state held behind the C-ABI handle (internal).
#pragma once

#include "common.cuh"

namespace tnr {

// leg labels of the contraction networks
enum { La = 0, Lb, Lc, Ld, Le, Lf, Lg, Lh, Li, Lj, Lk, Ll, Lm, Ln, Lo, Lp, Lq, Lr, Ls, Lt, Lu, Lv, Lw, Lx, Ly, Lz };

std::vector<double> dvec_to_host(Ctx& c, const double* d, int64_t n);
// T[..., i_leg, ...] *= v[i_leg]
void scale_leg(Ctx& c, DT& T, int leg, const double* v);

// Finalizer selected for finalize!/run! (Finalizer objects of src/utility/finalize.jl)
enum { FINALIZER_DEFAULT = 0, FINALIZER_TWO_BY_TWO = 1 };

// Split-precision runs compute their first coarse-graining steps in FP64 while the bond
// dimension is still growing (every input leg below chi): the norm of step i enters the
// free energy with weight 2^-i (8^-i in 3D), so the first three 2D steps (the first 3D
// step) carry 7/8 of it, while their tensors are still small.  A step whose input has
// reached chi runs split from the start.
#ifndef TNR_SPLIT_FP64_STEPS_2D
#define TNR_SPLIT_FP64_STEPS_2D 3
#endif
#ifndef TNR_SPLIT_FP64_STEPS_3D
#define TNR_SPLIT_FP64_STEPS_3D 1
#endif
// 2D steps at chi at or below this run in FP64 in a split-precision solve (split_step_in_fp64)
#ifndef TNR_SPLIT_MIN_CHI
#define TNR_SPLIT_MIN_CHI 16
#endif
int split_fp64_steps(int kind);
bool split_step_in_fp64(int kind, int64_t step, const int64_t* dims, int nlegs, int chi);

// switches a split-precision context to FP64 for one scope
struct PrecisionScope {
    Ctx& c;
    int saved;
    PrecisionScope(Ctx& ctx, bool fp64) : c(ctx), saved(ctx.precision) {
        if (fp64) c.precision = TNR_PREC_F64;
    }
    ~PrecisionScope() { c.precision = saved; }
    PrecisionScope(const PrecisionScope&) = delete;
    PrecisionScope& operator=(const PrecisionScope&) = delete;
};

struct Scheme {
    int kind = 0;
    std::unique_ptr<Ctx> ctx;
    DT T;
    DT S1, S2;                     // BTRG diagonal bond tensors
    DT I11, I12, I2;               // ImpurityHOTRG: +1 / -1 first-order and second-order impurity tensors
    DT site[4];                    // ImpurityTRG: impurity tensors on the four plaquette sites
    DT C1, C2, Cf;                 // CorrelationHOTRG: the two first-order impurities, then the merged one
    int corr_dist = 0;             // CorrelationHOTRG: the impurities merge at step corr_dist (2^dist apart)
    int finalizer = FINALIZER_DEFAULT;
    double btrg_k = -0.5;
    int64_t steps = 0;
    // run!() folds each step's normalisation into the next step: finalize! leaves T unscaled
    // and `pending` points at its norm n on the device; the next step's decompositions divide
    // their singular values by |n| (and HOTRG's permutes read T scaled), so the chi^4 tensor is
    // never rescaled in a pass of its own.  The last norm is applied when run!() ends.
    const double* pending = nullptr;
    int64_t max_slice_entries = int64_t(1) << 31;   // HOTRG_3D slicing budget (entries)
    std::vector<double> last_vals; // kept singular values / eigenvalues of the last step
    std::vector<int> last_counts;
    std::vector<double> last_eps;  // (eps, eps') pairs of the last step
    std::string err;

    // d_corr: CorrelationHOTRG's three norms of the step (device, may be null)
    void step(int chi, double* d_corr = nullptr);
    std::vector<double> run_correlation(int chi, int maxiter);   // three norms per step
    void finalize_async(double* d_norm, bool scale = true);
    bool folds_normalisation() const;
    double finalize();
    std::vector<double> run(int chi, int maxiter, bool finalize_beginning);
    // ImpurityHOTRG: the four trace norms (pure, +1, -1, second order) into d4[0..3]; every
    // tensor is divided by the pure norm
    void finalize_impurity_async(double* d4);
    // ImpurityTRG: the pure trace norm and the plaquette norm of the four impurities into d2[0..1]
    void finalize_impurity_trg_async(double* d2);
    int norms_per_entry() const { return kind == TNR_IMPURITY_HOTRG ? 4 : kind == TNR_IMPURITY_TRG ? 2 : 1; }
    void finalize_multi_async(double* d);
    std::vector<double> run_impurity(int chi, int maxiter, bool finalize_beginning);   // norms_per_entry() each
    void record(const TsvdOut& r);

    // finalizers on the fixed-point tensor (src/utility/cft.jl, src/utility/finalize.jl:17-41)
    void finalize_two_by_two_async(double* d_norm);      // n^(1/4) of the 2 x 2 plaquette; T /= it
    void transfer_eigvals(int unitcell, std::vector<double>& re, std::vector<double>& im);
    void gu_wen(double* x1, double* x2);
    double central_charge(double n);
};

// run!() of fresh TRG/BTRG schemes with equal kind, dims and k in lockstep on `c`;
// norms[b] receives member b's norms and every member is left in its final state
void run_group(Ctx& c, const std::vector<Scheme*>& members, int chi, int maxiter, bool finalize_beginning,
               std::vector<std::vector<double>>& norms);

}  // namespace tnr
