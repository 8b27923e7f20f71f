// Scheme state held behind the C-ABI handle (internal).
#pragma once

#include "common.cuh"

namespace tnr {

struct Scheme {
    int kind = 0;
    std::unique_ptr<Ctx> ctx;
    DT T;
    DT S1, S2;                     // BTRG diagonal bond tensors
    double btrg_k = -0.5;
    int64_t steps = 0;
    int64_t max_slice_entries = int64_t(1) << 31;   // HOTRG_3D slicing budget (entries)
    std::vector<double> last_vals; // kept singular values / eigenvalues of the last step
    std::vector<int> last_counts;
    std::vector<double> last_eps;  // (eps, eps') pairs of the last step
    std::string err;

    void step(int chi);
    void finalize_async(double* d_norm);
    double finalize();
    std::vector<double> run(int chi, int maxiter, bool finalize_beginning);
    void record(const TsvdOut& r);
};

// run!() of fresh TRG/BTRG schemes with equal kind, dims and k in lockstep on `c`;
// norms[b] receives member b's norms and every member is left in its final state
void run_group(Ctx& c, const std::vector<Scheme*>& members, int chi, int maxiter, bool finalize_beginning,
               std::vector<std::vector<double>>& norms);

}  // namespace tnr
