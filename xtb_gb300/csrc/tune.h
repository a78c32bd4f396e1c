// Per-device choices between kernel forms, measured by the engine's own autotuner.
//
// Two decisions of the single point depend on the matrix size and on the device: which
// tridiagonalisation runs (the row-by-row cooperative form, whose per-column vector work is
// cheap for small matrices, or the upper-triangle form with 4/3 n^3 flops), and from which size
// the back-transformation of the eigenvectors runs in the compact-WY form (FP64: column strips in
// one launch; split precision: tensor-core GEMMs per block) instead of one warp per vector.  Until `autotune` has run on a
// device the defaults below (measured once on GB300) apply; afterwards the engine uses the
// device's measured crossovers.
#pragma once
#include <vector>

namespace xg {

struct Tuned {
    int sytrd_sym_min = 1 << 30;    // AOs from which the upper-triangle tridiagonalisation runs
                                    // (never by default: on GB300 the row form measured faster up
                                    // to 1024 AOs, its per-column latency being lower)
    int blocked_min_fp64 = 300;     // AOs from which the compact-WY back-transformation runs
                                    // (FP64 column strips)
    int blocked_min_split = 1500;   // AOs from which split mode runs it as tensor-core GEMMs
                                    // (below, split mode takes the faster FP64 form)
    int level = 0;                  // 0: defaults, 1: measured on this device
    double seconds = 0.0;           // time the measurement took
    // measurements: (n, row form ms, upper-triangle form ms) and
    // (n, warp form ms, blocked FP64 ms, blocked split ms)
    std::vector<double> sytrd_rows, backtr_rows;
};

// the current device's choices
Tuned tuned();
// measure the crossovers on the current device (once; later calls return the kept choices)
Tuned autotune();
// CUDA-event time (ms, best of `reps`, the matrix copy included) of one tridiagonalisation of a
// random symmetric n x n matrix: form 0 row form, 1 upper-triangle form, -1 the tuned choice;
// max_blocks > 0 caps the cooperative grid
double time_sytrd(int n, int form, int max_blocks, int reps);
// compact-WY back-transformation (FP64 strips, or split products with slices > 0) against the
// warp-per-vector form on the first ncol columns of a random n x n matrix, Q from tridiagonalising
// a random symmetric matrix: out[0] max |difference| / max |Q Y|, out[1] and out[2] their ms
void check_backtransform(int n, int ncol, int slices, double* out);
// replace the current device's choices (level 1; for tests that pin a form)
void set_tuned(int sytrd_sym_min, int blocked_min_fp64, int blocked_min_split);
// back-transformation threshold for a precision (0 FP64, 1 split)
int tuned_blocked_min(int precision);
// tridiagonalisation threshold
int tuned_sytrd_sym_min();

}  // namespace xg
