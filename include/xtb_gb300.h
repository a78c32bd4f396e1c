/*
 * xtb_gb300.h -- engine extensions of libxtb_gb300.so beyond the reference C API.
 *
 * These entry points have no counterpart in the reference's include/xtb.h; they
 * expose information the GPU engine has and that tests, benchmarks and
 * serving layers need.  Same conventions as xtb.h: errors go to the
 * environment, NULL environment is a no-op, output arrays are caller-owned.
 */
#pragma once
#include "xtb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Number of CUDA devices visible to the engine (0 if none). */
extern int xtbgb_deviceCount(void);

/* SCC iterations of the last single point and whether it converged (1/0). */
extern void xtbgb_getIterations(xtb_TEnvironment env, xtb_TResults res, int* iterations, int* converged);

/* Energy decomposition of the last single point, Hartree (gap in eV):
 * parts[0] electronic (incl. three-body dispersion), [1] repulsion, [2] isotropic ES,
 * [3] anisotropic ES, [4] anisotropic XC, [5] dispersion, [6] three-body dispersion,
 * [7] HOMO-LUMO gap (eV). */
extern void xtbgb_getEnergyParts(xtb_TEnvironment env, xtb_TResults res, double* parts);

/* Shell charges[nshell] and cumulative atomic multipoles dipm[natoms][3],
 * qp[natoms][6] (packed xx, xy, yy, xz, yz, zz) of the last single point. */
extern void xtbgb_getShellCharges(xtb_TEnvironment env, xtb_TResults res, double* qsh);
extern void xtbgb_getMultipoles(xtb_TEnvironment env, xtb_TResults res, double* dipm, double* qp);

/* Device time (ms) of the last single point per engine phase, measured with CUDA
 * events on the engine's stream.  ms[0..11] = setup, integrals, cholesky, hbuild,
 * stdform, sytrd, trieig, backtransform, density, popmix, gradient, total. */
extern void xtbgb_getPhaseTimes(xtb_TEnvironment env, xtb_TResults res, double* ms);

/* Host<->device traffic of the last single point: bytes[0] host->device, bytes[1] device->host,
 * bytes[2] number of device kernels the single point launched. */
extern void xtbgb_getTransferBytes(xtb_TEnvironment env, xtb_TResults res, long long* bytes);

/* Whether the engine keeps orbital data (MO coefficients, density, overlap) on the host after a
 * single point; needed by xtb_getOrbitalCoefficients.  Default 1 (as the reference). */
extern void xtbgb_setKeepOrbitals(xtb_TEnvironment env, xtb_TCalculator calc, int keep);

/* Precision of the calculator's dense products: split = 0 (default) keeps every product in
 * FP64; split = 1 computes the back-transformation C = X Z, the density P = C f C^T and the
 * energy-weighted density as split-precision products on the BF16 tensor cores with `slices`
 * (4..7) digits of 8 bits per operand (5: about 2^-40 relative error per product term).  The
 * Cholesky factorisation, the reduction to standard form and the eigensolver stay FP64. */
extern void xtbgb_setPrecision(xtb_TEnvironment env, xtb_TCalculator calc, int split, int slices);

/* AO count from which the eigenvector back-transformation runs as blocked compact-WY products
 * (blocks of 128 reflectors) instead of one warp per eigenvector.  -1 (default) picks it by
 * precision: 1500 AOs for FP64, 1000 for split precision. */
extern void xtbgb_setBlockedBacktransform(xtb_TEnvironment env, xtb_TCalculator calc, int nao_min);

/* Measured FP64 throughput of device 0 in TFLOP/s (roofline denominator for FP64 kernels): the
 * largest of two FMA-throughput probes and the engine's own FP64 GEMM at 4096^3; returns 0 when
 * no device is present. */
extern double xtbgb_fp64PeakTflops(void);

/* Restart file of the reference (xtbrestart, src/restart.f90): a Fortran unformatted
 * sequential file holding the shell charges and, for GFN2, the atomic dipole and quadrupole
 * moments of the last single point on `res`.  xtbgb_writeRestart writes it (0 on error, reported
 * on env).  xtbgb_readRestart loads it into `res`, so that the next xtb_singlepoint on `res`
 * starts from it (the reference's warm start); it returns 1 when the file matched the molecule,
 * 0 otherwise, with the reference's warnings on env (a missing file is silently 0). */
extern int xtbgb_writeRestart(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TResults res, const char* filename);
extern int xtbgb_readRestart(xtb_TEnvironment env, xtb_TMolecule mol, xtb_TResults res, const char* filename);

/* External point charges with explicit hardness values (bohr, e; hardness in Eh).  The
 * reference's C API (xtb_setExternalCharges) takes each charge's hardness from an element
 * number; its Fortran calculator also accepts the hardness directly (calc%pcem%gam, used with
 * 999 for bare point charges in test/unit/test_gfn2.f90:500-520), which this call exposes.
 * Replaces earlier external charges on the calculator; errors as xtb_setExternalCharges. */
extern void xtbgb_setExternalChargesHardness(xtb_TEnvironment env, xtb_TCalculator calc, int n,
                                             const double* charges, const double* positions,
                                             const double* hardness);

/* Implicit solvent of the last single point (an xtb_setSolvent calculator): parts[0..4] = free
 * energy of solvation (contained in the total energy), its Born part (without the H-bond term),
 * the H-bond correction, the surface term and the constant shift, all in Hartree at the final
 * charges (getEnergyParts, src/solv/gbsa.f90:552-596; the reference keeps them in
 * scc_results%g_solv / g_born / g_hb / g_sasa / g_shift, src/scf_module.F90:906-912, without a C
 * getter: xtb_getSolvationEnergy serves only CPCM-X, include/xtb.h:276-280).  Returns 1 when the
 * single point had a solvent, else 0 (parts then zero). */
extern int xtbgb_getSolvationEnergyParts(xtb_TEnvironment env, xtb_TResults res, double* parts);

/* Salt screening of the GBSA kernel (Debye-Hueckel; TSolvInput%ionStrength / %ionRad,
 * src/solv/input.F90, src/solv/gbsa.f90:296-309, exercised by test/unit/test_gfn2.f90:310-381;
 * the reference C API has no setter): ion strength in mol/L (0 switches it off) and ion radius
 * in Bohr.  Kept across xtb_setSolvent calls on the calculator; needs the "gbsa" model. */
extern void xtbgb_setSolventSalt(xtb_TEnvironment env, xtb_TCalculator calc, double ion_strength,
                                 double ion_rad);

/* Born kernel of the solvent set on the calculator: 0 Still (with the GBSA parameter sets), 1 P16
 * (with the ALPB sets).  xtb_setSolvent ties the kernel to the model ("gbsa": Still, "alpb": P16);
 * TSolvInput%kernel (src/solv/input.F90) decouples them, as test/unit/test_gfn2.f90:745-828 does
 * with the ALPB correction on the Still kernel.  Call after xtb_setSolvent. */
extern void xtbgb_setSolventKernel(xtb_TEnvironment env, xtb_TCalculator calc, int kernel);

/* Autotuner (no counterpart in the reference).  Two choices of the single point depend on the
 * matrix size and the device: the form of the tridiagonalisation (row by row, or the
 * upper-triangle form with 4/3 n^3 flops) and the form of the eigenvector back-transformation
 * (one warp per vector, or compact-WY GEMMs; FP64 and split precision apart).  xtbgb_autotune
 * times both forms of each on synthetic matrices of the current device (a few seconds, once per
 * device and process; later calls return the kept choices) and the engine uses the measured
 * crossovers from then on.  out[nout] receives: [0] AOs from which the upper-triangle
 * tridiagonalisation runs, [1] AOs from which the blocked back-transformation runs in FP64,
 * [2] the same in split precision, [3] seconds taken, [4] R, then R rows (n, row form ms,
 * upper-triangle form ms), then R2, then R2 rows (n, warp form ms, blocked FP64 ms, blocked
 * split ms).  Returns the number of values written (0 on error, reported on env). */
extern int xtbgb_autotune(xtb_TEnvironment env, double* out, int nout);
/* CUDA-event time in ms (best of reps, a device-to-device copy of the matrix included) of one
 * tridiagonalisation of a random symmetric n x n matrix (3 <= n <= 8192) on the current device:
 * form 0 the row form, 1 the upper-triangle form, -1 the tuned choice; max_blocks > 0 caps the
 * cooperative grid.  Returns -1 on error (reported on env). */
extern double xtbgb_sytrdMs(xtb_TEnvironment env, int n, int form, int max_blocks, int reps);
/* The eigenvector back-transformation Z = Q Y of the first ncol (1..n) columns of a random
 * n x n matrix (3 <= n <= 8192; Q from tridiagonalising a random symmetric matrix) by the
 * compact-WY form (slices 0: FP64 column strips, 1..8: split-precision products with that many
 * bf16 digits) against the one-warp-per-vector form: out[0] max |difference| / max |Z|, out[1]
 * and out[2] the two forms' CUDA-event ms.  Returns 0, or 1 on error (reported on env). */
extern int xtbgb_backtransformCheck(xtb_TEnvironment env, int n, int ncol, int slices, double* out);
/* The current device's choices: out[0..2] as above, out[3] 1 when measured, 0 for defaults. */
extern void xtbgb_getTuning(xtb_TEnvironment env, double* out);
/* Pin the current device's choices (sizes in AOs; for tests and for callers with their own
 * measurements). */
extern void xtbgb_setTuning(xtb_TEnvironment env, int sytrd_sym_min, int blocked_min_fp64, int blocked_min_split);

/* The three figures behind xtbgb_fp64PeakTflops, measured anew (TFLOP/s): out[0] FMA chains with
 * uniform operands, out[1] GEMM-style accumulator chains, out[2] FP64 GEMM C = A B at 4096^3. */
extern void xtbgb_fp64PeakDetail(double* out);

/* Dependent-operation latency of device 0 in clock cycles, measured with one warp:
 * cycles[0] FP64 FMA, [1] FP64 add, [2] FP64 multiply, [3] FP64 divide, [4] FP32 FMA
 * (all 0 when no device is present). */
extern void xtbgb_fp64LatencyCycles(double* cycles);

/* Check the FP64 reciprocal used on the dependent chains of inverse iteration (an FP32 seed
 * refined by one third-order Newton step) against the FP64 division on device 0: out[0] the
 * largest difference in units of the last place, out[1] the number of values checked
 * (+-(1 + t 2^-20) 2^k, k in [-1000, 1000]).  Returns 0 on success. */
extern int xtbgb_reciprocalCheck(double* out);

/* Check and time the split-precision GEMM (FP64 results from BF16 tensor-core products of
 * fixed-point digit slices) against the FP64 GEMM on seeded random M x K and K x N matrices
 * with entries uniform(-1,1) * 2^-e, e in [0, exp_range].  out[0] max |dC| / (|A||B|),
 * out[1] max |dC| / max |C|, out[2] split ms, out[3] FP64 ms, out[4] split TFLOP/s, out[5] FP64
 * TFLOP/s.  slices 4..7.  Returns 0 on success. */
extern int xtbgb_splitGemmCheck(int M, int N, int K, int slices, int seed, int exp_range, double* out);

/* ---- Batched single points (no counterpart in the reference: the reference API runs one
 * molecule per call).  Many molecules of uneven size are solved together on the device, one
 * thread block per molecule with its whole SCC state resident; molecules above 512 AOs (or
 * whose SCC outgrows the batched mixing history) run on the plain per-molecule GPU engine.
 * GFN2-xTB, gas phase; results are reported per molecule in input order. */
typedef struct _xtbgb_TBatch* xtbgb_TBatch;

/* natoms[nmol]; numbers[sum natoms] and positions[sum natoms][3] (Bohr) concatenated in
 * molecule order; charges[nmol] and uhf[nmol] may be NULL (neutral, closed shell). */
extern xtbgb_TBatch xtbgb_newBatch(xtb_TEnvironment env, int nmol, const int* natoms, const int* numbers,
                                   const double* positions, const double* charges, const int* uhf);
extern void xtbgb_delBatch(xtbgb_TBatch* batch);
/* All single points with one set of settings (accuracy, electronic temperature in K, maximum
 * SCC iterations, clamped as by xtb_setAccuracy / xtb_setElectronicTemp / xtb_setMaxIter);
 * gradient != 0 also computes gradients.  Failed or unconverged molecules raise one error on
 * the environment; their results are still filled. */
extern void xtbgb_batchSinglepoint(xtb_TEnvironment env, xtbgb_TBatch batch, double accuracy, double etemp,
                                   int maxiter, int gradient);
extern void xtbgb_batchGetEnergies(xtb_TEnvironment env, xtbgb_TBatch batch, double* energies);   /* [nmol] */
extern void xtbgb_batchGetGradients(xtb_TEnvironment env, xtbgb_TBatch batch, double* gradients); /* [N][3] */
extern void xtbgb_batchGetCharges(xtb_TEnvironment env, xtbgb_TBatch batch, double* charges);     /* [N] */
extern void xtbgb_batchGetDipoles(xtb_TEnvironment env, xtbgb_TBatch batch, double* dipoles);     /* [nmol][3] */
/* [nmol][8], the same parts as xtbgb_getEnergyParts */
extern void xtbgb_batchGetEnergyParts(xtb_TEnvironment env, xtbgb_TBatch batch, double* parts);
/* per molecule: SCC iterations, converged (1/0), status (0 ok, 1 not converged, 2 overlap not
 * positive definite, 3 non-finite energy), engine (0 batched, 1 plain); any pointer may be NULL */
extern void xtbgb_batchGetStatus(xtb_TEnvironment env, xtbgb_TBatch batch, int* iterations, int* converged,
                                 int* status, int* engine);
/* times[0] device ms (CUDA events around the batched kernels, plus plain-engine device time),
 * times[1] wall ms of the call; counts[0] host->device bytes, [1] device->host bytes,
 * [2] kernel launches, [3] molecules run on the plain engine. */
extern void xtbgb_batchGetStats(xtb_TEnvironment env, xtbgb_TBatch batch, double* times, long long* counts);
/* number of AOs of every molecule [nmol] */
extern void xtbgb_batchNao(xtb_TEnvironment env, xtbgb_TBatch batch, int* nao);

/* ---- Request loop (no counterpart in the reference).  A server owns a resident pool of
 * molecules on the device (HBM budget pool_gib GiB, at most max_slots molecules) that is
 * advanced iters_per_step SCC iterations per step with continuous batching: requests that
 * arrive while others run join the next step.  Molecules above 512 AOs run on
 * plain_workers concurrent plain-engine workers.  Submit and wait may be called from any
 * thread, each thread with its own environment. */
typedef struct _xtbgb_TServer* xtbgb_TServer;

extern xtbgb_TServer xtbgb_newServer(xtb_TEnvironment env, double pool_gib, int max_slots, int plain_workers,
                                     int iters_per_step, double accuracy, double etemp, int maxiter);
/* As xtbgb_newServer; split = 1 runs the plain-engine workers with split-precision products
 * (xtbgb_setPrecision semantics, `slices` digits); pool_max_nao (1..512, <= 0 for 512) is the
 * largest molecule in AOs the resident pool takes, larger ones go to the plain-engine workers;
 * coop_blocks > 0 caps the blocks of a worker's cooperative tridiagonalisation (0: one per SM),
 * so that the workers' single points can share the SMs; coop_blocks = -D caps it at one block per
 * D AOs of the request (at least 8). */
extern xtbgb_TServer xtbgb_newServerEx(xtb_TEnvironment env, double pool_gib, int max_slots, int plain_workers,
                                       int iters_per_step, double accuracy, double etemp, int maxiter, int split,
                                       int slices, int pool_max_nao, int coop_blocks);
/* Finishes all submitted work, then frees the server. */
extern void xtbgb_delServer(xtbgb_TServer* server);
/* Queue one GFN2-xTB single point (positions [natoms][3] Bohr); returns the request id, or
 * -1 with an error on the environment. */
extern long long xtbgb_serverSubmit(xtb_TEnvironment env, xtbgb_TServer server, int natoms, const int* numbers,
                                    const double* positions, double charge, int uhf, int gradient);
/* Wait for request `id` (timeout in seconds, < 0 waits forever).  Returns 1 and fills the
 * outputs when the request is done, 0 on timeout.  energy[1]; gradient[natoms][3] and
 * charges[natoms] may be NULL; info[12]: SCC iterations, converged, status, engine
 * (0 pool, 1 plain), submit / start / done times (s since the server started), dipole[3],
 * number of AOs, device ms of the tridiagonalisations (plain engine only).
 * A failed or unconverged request also raises an error on the environment. */
extern int xtbgb_serverWait(xtb_TEnvironment env, xtbgb_TServer server, long long id, double timeout,
                            double* energy, double* gradient, double* charges, double* info);
/* stats[11]: completed, run on the plain engine, pool steps, pool busy seconds, peak resident
 * molecules, requests re-run on the plain engine, host->device bytes, device->host bytes,
 * kernel launches, device ms of the pool's SCC kernel, algorithmic FP64 flops of the pool's
 * SCC iterations (n^3 + 4/3 n^3 + 2 n^3 + n^3 + 2 n^2 k per molecule and iteration). */
extern void xtbgb_serverStats(xtb_TEnvironment env, xtbgb_TServer server, double* stats);
/* Test hook (no counterpart in the reference), host side only: the next `count` admissions to
 * the resident pool fail as if the device had run out of memory.  Each such request completes
 * with status 3 and the error on the waiting environment; the pool keeps serving the others. */
extern void xtbgb_serverInjectAdmissionFailures(xtb_TEnvironment env, xtbgb_TServer server, int count);

/* Repulsion energy and gradient of one molecule, computed from and into DEVICE memory
 * without allocating anything.  No counterpart in the reference: it exists for callers
 * that own all device memory themselves (a serving loop that admits work against a fixed
 * HBM budget, an MD code keeping coordinates resident), for which a library-side
 * cudaMalloc would break the budget and a cudaFree would stall the whole device.
 *   numbers[natoms] (int), positions[natoms][3] (Bohr)  -> device inputs
 *   energy[1] (Hartree), gradient[natoms][3] (Hartree/Bohr) -> device outputs, overwritten
 *   stream: a cudaStream_t (NULL = legacy default stream); the call only enqueues work.
 * The scratch is a static device array sized for natoms <= 8192; larger inputs are
 * rejected.  The first call on each device looks up that array (cudaGetSymbolAddress) and
 * should come before any stream capture.  Calls that overlap in time share the scratch
 * and race: serialise them.  Returns 0 on success, else a nonzero code with a message in
 * errbuf[errlen] (errbuf may be NULL).  The atomic numbers are device data and are not checked on
 * the host: an element outside 1..86 still returns 0, with a NaN energy.  The scratch address is
 * cached per device at the first call; resetting the device (cudaDeviceReset) between calls is
 * not supported. */
extern int xtbgb_repulsionNoAlloc(int natoms, const int* numbers, const double* positions, double* energy,
                                  double* gradient, void* stream, char* errbuf, int errlen);

#ifdef __cplusplus
}
#endif
