! ISO_C_BINDING interface of libxtb_gb300.so for Fortran hosts.
!
! Binds the C API declared in xtb.h (the same symbols as the reference's
! include/xtb.h:71-310) and every extension declared in xtb_gb300.h.  Handles are
! opaque type(c_ptr); arrays are passed by address in Fortran (column-major)
! order, so positions(3, natoms) and gradient(3, natoms) map directly onto the
! C layout [natoms][3].  Arguments the C side accepts as NULL are optional here
! (absent = NULL); the allocation-free repulsion takes device addresses as
! type(c_ptr).  Link with -lxtb_gb300.
module xtb_gb300_api
   use, intrinsic :: iso_c_binding, only : c_ptr, c_int, c_double, c_bool, c_char, c_long_long
   implicit none
   private

   public :: xtb_getAPIVersion, xtb_newEnvironment, xtb_delEnvironment, xtb_checkEnvironment
   public :: xtb_getError, xtb_setVerbosity
   public :: xtb_newMolecule, xtb_delMolecule, xtb_updateMolecule
   public :: xtb_newCalculator, xtb_delCalculator, xtb_loadGFN2xTB
   public :: xtb_setAccuracy, xtb_setMaxIter, xtb_setElectronicTemp
   public :: xtb_singlepoint, xtb_newResults, xtb_delResults
   public :: xtb_getEnergy, xtb_getGradient, xtb_getCharges, xtb_getDipole
   public :: xtbgb_newBatch, xtbgb_delBatch, xtbgb_batchSinglepoint
   public :: xtbgb_batchGetEnergies, xtbgb_batchGetGradients, xtbgb_batchGetCharges
   public :: xtb_showEnvironment, xtb_setOutput, xtb_releaseOutput, xtb_loadGFN0xTB
   public :: xtb_loadGFN1xTB, xtb_loadGFNFF, xtb_setSolvent, xtb_releaseSolvent
   public :: xtb_setExternalCharges, xtb_releaseExternalCharges, xtb_hessian, xtb_cpcmx_calc
   public :: xtb_copyResults, xtb_getSolvationEnergy, xtb_getPCGradient, xtb_getVirial
   public :: xtb_getBondOrders, xtb_getNao, xtb_getOrbitalEigenvalues, xtb_getOrbitalOccupations
   public :: xtb_getOrbitalCoefficients, xtbgb_deviceCount, xtbgb_getIterations
   public :: xtbgb_getEnergyParts, xtbgb_getShellCharges, xtbgb_getMultipoles, xtbgb_getPhaseTimes
   public :: xtbgb_getTransferBytes, xtbgb_setKeepOrbitals, xtbgb_setPrecision
   public :: xtbgb_setBlockedBacktransform, xtbgb_fp64PeakTflops, xtbgb_writeRestart
   public :: xtbgb_readRestart, xtbgb_setExternalChargesHardness, xtbgb_getSolvationEnergyParts
   public :: xtbgb_setSolventSalt, xtbgb_setSolventKernel, xtbgb_autotune, xtbgb_sytrdMs
   public :: xtbgb_backtransformCheck
   public :: xtbgb_getTuning, xtbgb_setTuning, xtbgb_fp64PeakDetail, xtbgb_fp64LatencyCycles
   public :: xtbgb_reciprocalCheck, xtbgb_splitGemmCheck, xtbgb_batchGetDipoles
   public :: xtbgb_batchGetEnergyParts, xtbgb_batchGetStatus, xtbgb_batchGetStats, xtbgb_batchNao
   public :: xtbgb_newServer, xtbgb_newServerEx, xtbgb_delServer, xtbgb_serverSubmit
   public :: xtbgb_serverWait, xtbgb_serverStats, xtbgb_serverInjectAdmissionFailures
   public :: xtbgb_repulsionNoAlloc

   interface
      integer(c_int) function xtb_getAPIVersion() bind(C, name="xtb_getAPIVersion")
         import :: c_int
      end function

      type(c_ptr) function xtb_newEnvironment() bind(C, name="xtb_newEnvironment")
         import :: c_ptr
      end function

      subroutine xtb_delEnvironment(env) bind(C, name="xtb_delEnvironment")
         import :: c_ptr
         type(c_ptr), intent(inout) :: env
      end subroutine

      integer(c_int) function xtb_checkEnvironment(env) bind(C, name="xtb_checkEnvironment")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
      end function

      subroutine xtb_getError(env, buffer, buffersize) bind(C, name="xtb_getError")
         import :: c_ptr, c_char, c_int
         type(c_ptr), value :: env
         character(kind=c_char), intent(out) :: buffer(*)
         integer(c_int), intent(in) :: buffersize
      end subroutine

      subroutine xtb_setVerbosity(env, verbosity) bind(C, name="xtb_setVerbosity")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         integer(c_int), value :: verbosity
      end subroutine

      type(c_ptr) function xtb_newMolecule(env, natoms, numbers, positions, charge, uhf, lattice, periodic) &
            bind(C, name="xtb_newMolecule")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: env
         integer(c_int), intent(in) :: natoms
         integer(c_int), intent(in) :: numbers(*)
         real(c_double), intent(in) :: positions(3, *)
         real(c_double), intent(in), optional :: charge
         integer(c_int), intent(in), optional :: uhf
         type(c_ptr), value :: lattice
         type(c_ptr), value :: periodic
      end function

      subroutine xtb_delMolecule(mol) bind(C, name="xtb_delMolecule")
         import :: c_ptr
         type(c_ptr), intent(inout) :: mol
      end subroutine

      subroutine xtb_updateMolecule(env, mol, positions, lattice) bind(C, name="xtb_updateMolecule")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, mol
         real(c_double), intent(in) :: positions(3, *)
         type(c_ptr), value :: lattice
      end subroutine

      type(c_ptr) function xtb_newCalculator() bind(C, name="xtb_newCalculator")
         import :: c_ptr
      end function

      subroutine xtb_delCalculator(calc) bind(C, name="xtb_delCalculator")
         import :: c_ptr
         type(c_ptr), intent(inout) :: calc
      end subroutine

      subroutine xtb_loadGFN2xTB(env, mol, calc, filename) bind(C, name="xtb_loadGFN2xTB")
         import :: c_ptr
         type(c_ptr), value :: env, mol, calc
         type(c_ptr), value :: filename
      end subroutine

      subroutine xtb_setAccuracy(env, calc, accuracy) bind(C, name="xtb_setAccuracy")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, calc
         real(c_double), value :: accuracy
      end subroutine

      subroutine xtb_setMaxIter(env, calc, iterations) bind(C, name="xtb_setMaxIter")
         import :: c_ptr, c_int
         type(c_ptr), value :: env, calc
         integer(c_int), value :: iterations
      end subroutine

      subroutine xtb_setElectronicTemp(env, calc, temperature) bind(C, name="xtb_setElectronicTemp")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, calc
         real(c_double), value :: temperature
      end subroutine

      subroutine xtb_singlepoint(env, mol, calc, res) bind(C, name="xtb_singlepoint")
         import :: c_ptr
         type(c_ptr), value :: env, mol, calc, res
      end subroutine

      type(c_ptr) function xtb_newResults() bind(C, name="xtb_newResults")
         import :: c_ptr
      end function

      subroutine xtb_delResults(res) bind(C, name="xtb_delResults")
         import :: c_ptr
         type(c_ptr), intent(inout) :: res
      end subroutine

      subroutine xtb_getEnergy(env, res, energy) bind(C, name="xtb_getEnergy")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, res
         real(c_double), intent(out) :: energy
      end subroutine

      subroutine xtb_getGradient(env, res, gradient) bind(C, name="xtb_getGradient")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, res
         real(c_double), intent(out) :: gradient(3, *)
      end subroutine

      subroutine xtb_getCharges(env, res, charges) bind(C, name="xtb_getCharges")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, res
         real(c_double), intent(out) :: charges(*)
      end subroutine

      subroutine xtb_getDipole(env, res, dipole) bind(C, name="xtb_getDipole")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, res
         real(c_double), intent(out) :: dipole(3)
      end subroutine

      type(c_ptr) function xtbgb_newBatch(env, nmol, natoms, numbers, positions, charges, uhf) &
            bind(C, name="xtbgb_newBatch")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: env
         integer(c_int), value :: nmol
         integer(c_int), intent(in) :: natoms(*), numbers(*)
         real(c_double), intent(in) :: positions(3, *)
         real(c_double), intent(in), optional :: charges(*)
         integer(c_int), intent(in), optional :: uhf(*)
      end function

      subroutine xtbgb_delBatch(batch) bind(C, name="xtbgb_delBatch")
         import :: c_ptr
         type(c_ptr), intent(inout) :: batch
      end subroutine

      subroutine xtbgb_batchSinglepoint(env, batch, accuracy, etemp, maxiter, gradient) &
            bind(C, name="xtbgb_batchSinglepoint")
         import :: c_ptr, c_double, c_int
         type(c_ptr), value :: env, batch
         real(c_double), value :: accuracy, etemp
         integer(c_int), value :: maxiter, gradient
      end subroutine

      subroutine xtbgb_batchGetEnergies(env, batch, energies) bind(C, name="xtbgb_batchGetEnergies")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, batch
         real(c_double), intent(out) :: energies(*)
      end subroutine

      subroutine xtbgb_batchGetGradients(env, batch, gradients) bind(C, name="xtbgb_batchGetGradients")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, batch
         real(c_double), intent(out) :: gradients(3, *)
      end subroutine

      subroutine xtbgb_batchGetCharges(env, batch, charges) bind(C, name="xtbgb_batchGetCharges")
         import :: c_ptr, c_double
         type(c_ptr), value :: env, batch
         real(c_double), intent(out) :: charges(*)
      end subroutine

      subroutine xtb_showEnvironment(env, message) bind(C, name="xtb_showEnvironment")
         import :: c_ptr, c_char
         type(c_ptr), value :: env
         character(kind=c_char), intent(in) :: message(*)
      end subroutine

      subroutine xtb_setOutput(env, filename) bind(C, name="xtb_setOutput")
         import :: c_ptr, c_char
         type(c_ptr), value :: env
         character(kind=c_char), intent(in) :: filename(*)
      end subroutine

      subroutine xtb_releaseOutput(env) bind(C, name="xtb_releaseOutput")
         import :: c_ptr
         type(c_ptr), value :: env
      end subroutine

      subroutine xtb_loadGFN0xTB(env, mol, calc, filename) bind(C, name="xtb_loadGFN0xTB")
         import :: c_ptr
         type(c_ptr), value :: env
         type(c_ptr), value :: mol
         type(c_ptr), value :: calc
         type(c_ptr), value :: filename
      end subroutine

      subroutine xtb_loadGFN1xTB(env, mol, calc, filename) bind(C, name="xtb_loadGFN1xTB")
         import :: c_ptr
         type(c_ptr), value :: env
         type(c_ptr), value :: mol
         type(c_ptr), value :: calc
         type(c_ptr), value :: filename
      end subroutine

      subroutine xtb_loadGFNFF(env, mol, calc, filename) bind(C, name="xtb_loadGFNFF")
         import :: c_ptr
         type(c_ptr), value :: env
         type(c_ptr), value :: mol
         type(c_ptr), value :: calc
         type(c_ptr), value :: filename
      end subroutine

      subroutine xtb_setSolvent(env, calc, solvent, state, temp, grid, model) bind(C, name="xtb_setSolvent")
         import :: c_ptr, c_char, c_int, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         character(kind=c_char), intent(in) :: solvent(*)
         integer(c_int), intent(in), optional :: state
         real(c_double), intent(in), optional :: temp
         integer(c_int), intent(in), optional :: grid
         character(kind=c_char), intent(in), optional :: model(*)
      end subroutine

      subroutine xtb_releaseSolvent(env, calc) bind(C, name="xtb_releaseSolvent")
         import :: c_ptr
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
      end subroutine

      subroutine xtb_setExternalCharges(env, calc, n, numbers, charges, positions) &
            bind(C, name="xtb_setExternalCharges")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         integer(c_int), intent(in) :: n
         integer(c_int), intent(in) :: numbers(*)
         real(c_double), intent(in) :: charges(*)
         real(c_double), intent(in) :: positions(3, *)
      end subroutine

      subroutine xtb_releaseExternalCharges(env, calc) bind(C, name="xtb_releaseExternalCharges")
         import :: c_ptr
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
      end subroutine

      subroutine xtb_hessian(env, mol, calc, res, hessian, atom_index_list, step_size, dipole_gradient, polarizability_gradient) &
            bind(C, name="xtb_hessian")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: mol
         type(c_ptr), value :: calc
         type(c_ptr), value :: res
         real(c_double), intent(out) :: hessian(*)
         type(c_ptr), value :: atom_index_list
         type(c_ptr), value :: step_size
         real(c_double), intent(out), optional :: dipole_gradient(*)
         type(c_ptr), value :: polarizability_gradient
      end subroutine

      subroutine xtb_cpcmx_calc(env, mol, calc, res) bind(C, name="xtb_cpcmx_calc")
         import :: c_ptr
         type(c_ptr), value :: env
         type(c_ptr), value :: mol
         type(c_ptr), value :: calc
         type(c_ptr), value :: res
      end subroutine

      type(c_ptr) function xtb_copyResults(res) bind(C, name="xtb_copyResults")
         import :: c_ptr
         type(c_ptr), value :: res
      end function

      subroutine xtb_getSolvationEnergy(env, res, energy) bind(C, name="xtb_getSolvationEnergy")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: energy
      end subroutine

      subroutine xtb_getPCGradient(env, res, gradient) bind(C, name="xtb_getPCGradient")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: gradient(3, *)
      end subroutine

      subroutine xtb_getVirial(env, res, virial) bind(C, name="xtb_getVirial")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: virial(3, 3)
      end subroutine

      subroutine xtb_getBondOrders(env, res, wbo) bind(C, name="xtb_getBondOrders")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: wbo(*)
      end subroutine

      subroutine xtb_getNao(env, res, nao) bind(C, name="xtb_getNao")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         integer(c_int), intent(out) :: nao
      end subroutine

      subroutine xtb_getOrbitalEigenvalues(env, res, emo) bind(C, name="xtb_getOrbitalEigenvalues")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: emo(*)
      end subroutine

      subroutine xtb_getOrbitalOccupations(env, res, focc) bind(C, name="xtb_getOrbitalOccupations")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: focc(*)
      end subroutine

      subroutine xtb_getOrbitalCoefficients(env, res, c) bind(C, name="xtb_getOrbitalCoefficients")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: c(*)
      end subroutine

      integer(c_int) function xtbgb_deviceCount() bind(C, name="xtbgb_deviceCount")
         import :: c_int
      end function

      subroutine xtbgb_getIterations(env, res, iterations, converged) bind(C, name="xtbgb_getIterations")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         integer(c_int), intent(out) :: iterations
         integer(c_int), intent(out) :: converged
      end subroutine

      subroutine xtbgb_getEnergyParts(env, res, parts) bind(C, name="xtbgb_getEnergyParts")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: parts(*)
      end subroutine

      subroutine xtbgb_getShellCharges(env, res, qsh) bind(C, name="xtbgb_getShellCharges")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: qsh(*)
      end subroutine

      subroutine xtbgb_getMultipoles(env, res, dipm, qp) bind(C, name="xtbgb_getMultipoles")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: dipm(3, *)
         real(c_double), intent(out) :: qp(6, *)
      end subroutine

      subroutine xtbgb_getPhaseTimes(env, res, ms) bind(C, name="xtbgb_getPhaseTimes")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: ms(*)
      end subroutine

      subroutine xtbgb_getTransferBytes(env, res, bytes) bind(C, name="xtbgb_getTransferBytes")
         import :: c_ptr, c_long_long
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         integer(c_long_long), intent(out) :: bytes(*)
      end subroutine

      subroutine xtbgb_setKeepOrbitals(env, calc, keep) bind(C, name="xtbgb_setKeepOrbitals")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         integer(c_int), value :: keep
      end subroutine

      subroutine xtbgb_setPrecision(env, calc, split, slices) bind(C, name="xtbgb_setPrecision")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         integer(c_int), value :: split
         integer(c_int), value :: slices
      end subroutine

      subroutine xtbgb_setBlockedBacktransform(env, calc, nao_min) &
            bind(C, name="xtbgb_setBlockedBacktransform")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         integer(c_int), value :: nao_min
      end subroutine

      real(c_double) function xtbgb_fp64PeakTflops() bind(C, name="xtbgb_fp64PeakTflops")
         import :: c_double
      end function

      integer(c_int) function xtbgb_writeRestart(env, mol, res, filename) bind(C, name="xtbgb_writeRestart")
         import :: c_int, c_ptr, c_char
         type(c_ptr), value :: env
         type(c_ptr), value :: mol
         type(c_ptr), value :: res
         character(kind=c_char), intent(in) :: filename(*)
      end function

      integer(c_int) function xtbgb_readRestart(env, mol, res, filename) bind(C, name="xtbgb_readRestart")
         import :: c_int, c_ptr, c_char
         type(c_ptr), value :: env
         type(c_ptr), value :: mol
         type(c_ptr), value :: res
         character(kind=c_char), intent(in) :: filename(*)
      end function

      subroutine xtbgb_setExternalChargesHardness(env, calc, n, charges, positions, hardness) &
            bind(C, name="xtbgb_setExternalChargesHardness")
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         integer(c_int), value :: n
         real(c_double), intent(in) :: charges(*)
         real(c_double), intent(in) :: positions(3, *)
         real(c_double), intent(in) :: hardness(*)
      end subroutine

      integer(c_int) function xtbgb_getSolvationEnergyParts(env, res, parts) &
            bind(C, name="xtbgb_getSolvationEnergyParts")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: res
         real(c_double), intent(out) :: parts(*)
      end function

      subroutine xtbgb_setSolventSalt(env, calc, ion_strength, ion_rad) bind(C, name="xtbgb_setSolventSalt")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         real(c_double), value :: ion_strength
         real(c_double), value :: ion_rad
      end subroutine

      subroutine xtbgb_setSolventKernel(env, calc, kernel) bind(C, name="xtbgb_setSolventKernel")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: calc
         integer(c_int), value :: kernel
      end subroutine

      integer(c_int) function xtbgb_autotune(env, out, nout) bind(C, name="xtbgb_autotune")
         import :: c_ptr, c_double, c_int
         type(c_ptr), value :: env
         real(c_double), intent(out) :: out(*)
         integer(c_int), value :: nout
      end function

      real(c_double) function xtbgb_sytrdMs(env, n, form, max_blocks, reps) bind(C, name="xtbgb_sytrdMs")
         import :: c_double, c_ptr, c_int
         type(c_ptr), value :: env
         integer(c_int), value :: n
         integer(c_int), value :: form
         integer(c_int), value :: max_blocks
         integer(c_int), value :: reps
      end function

      integer(c_int) function xtbgb_backtransformCheck(env, n, ncol, slices, out) &
            bind(C, name="xtbgb_backtransformCheck")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: env
         integer(c_int), value :: n
         integer(c_int), value :: ncol
         integer(c_int), value :: slices
         real(c_double), intent(out) :: out(*)
      end function

      subroutine xtbgb_getTuning(env, out) bind(C, name="xtbgb_getTuning")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         real(c_double), intent(out) :: out(*)
      end subroutine

      subroutine xtbgb_setTuning(env, sytrd_sym_min, blocked_min_fp64, blocked_min_split) &
            bind(C, name="xtbgb_setTuning")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         integer(c_int), value :: sytrd_sym_min
         integer(c_int), value :: blocked_min_fp64
         integer(c_int), value :: blocked_min_split
      end subroutine

      subroutine xtbgb_fp64PeakDetail(out) bind(C, name="xtbgb_fp64PeakDetail")
         import :: c_double
         real(c_double), intent(out) :: out(*)
      end subroutine

      subroutine xtbgb_fp64LatencyCycles(cycles) bind(C, name="xtbgb_fp64LatencyCycles")
         import :: c_double
         real(c_double), intent(out) :: cycles(*)
      end subroutine

      integer(c_int) function xtbgb_reciprocalCheck(out) bind(C, name="xtbgb_reciprocalCheck")
         import :: c_int, c_double
         real(c_double), intent(out) :: out(*)
      end function

      integer(c_int) function xtbgb_splitGemmCheck(m, n, k, slices, seed, exp_range, out) &
            bind(C, name="xtbgb_splitGemmCheck")
         import :: c_int, c_double
         integer(c_int), value :: m
         integer(c_int), value :: n
         integer(c_int), value :: k
         integer(c_int), value :: slices
         integer(c_int), value :: seed
         integer(c_int), value :: exp_range
         real(c_double), intent(out) :: out(*)
      end function

      subroutine xtbgb_batchGetDipoles(env, batch, dipoles) bind(C, name="xtbgb_batchGetDipoles")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: batch
         real(c_double), intent(out) :: dipoles(3, *)
      end subroutine

      subroutine xtbgb_batchGetEnergyParts(env, batch, parts) bind(C, name="xtbgb_batchGetEnergyParts")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: batch
         real(c_double), intent(out) :: parts(*)
      end subroutine

      subroutine xtbgb_batchGetStatus(env, batch, iterations, converged, status, engine) &
            bind(C, name="xtbgb_batchGetStatus")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: batch
         integer(c_int), intent(out), optional :: iterations(*)
         integer(c_int), intent(out), optional :: converged(*)
         integer(c_int), intent(out), optional :: status(*)
         integer(c_int), intent(out), optional :: engine(*)
      end subroutine

      subroutine xtbgb_batchGetStats(env, batch, times, counts) bind(C, name="xtbgb_batchGetStats")
         import :: c_ptr, c_double, c_long_long
         type(c_ptr), value :: env
         type(c_ptr), value :: batch
         real(c_double), intent(out) :: times(*)
         integer(c_long_long), intent(out) :: counts(*)
      end subroutine

      subroutine xtbgb_batchNao(env, batch, nao) bind(C, name="xtbgb_batchNao")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: batch
         integer(c_int), intent(out) :: nao(*)
      end subroutine

      type(c_ptr) function xtbgb_newServer(env, pool_gib, max_slots, plain_workers, iters_per_step, accuracy, etemp, maxiter) &
            bind(C, name="xtbgb_newServer")
         import :: c_ptr, c_double, c_int
         type(c_ptr), value :: env
         real(c_double), value :: pool_gib
         integer(c_int), value :: max_slots
         integer(c_int), value :: plain_workers
         integer(c_int), value :: iters_per_step
         real(c_double), value :: accuracy
         real(c_double), value :: etemp
         integer(c_int), value :: maxiter
      end function

      type(c_ptr) function xtbgb_newServerEx(env, pool_gib, max_slots, plain_workers, iters_per_step, accuracy, etemp, maxiter, split, slices, pool_max_nao, coop_blocks) &
            bind(C, name="xtbgb_newServerEx")
         import :: c_ptr, c_double, c_int
         type(c_ptr), value :: env
         real(c_double), value :: pool_gib
         integer(c_int), value :: max_slots
         integer(c_int), value :: plain_workers
         integer(c_int), value :: iters_per_step
         real(c_double), value :: accuracy
         real(c_double), value :: etemp
         integer(c_int), value :: maxiter
         integer(c_int), value :: split
         integer(c_int), value :: slices
         integer(c_int), value :: pool_max_nao
         integer(c_int), value :: coop_blocks
      end function

      subroutine xtbgb_delServer(server) bind(C, name="xtbgb_delServer")
         import :: c_ptr
         type(c_ptr), intent(inout) :: server
      end subroutine

      integer(c_long_long) function xtbgb_serverSubmit(env, server, natoms, numbers, positions, charge, uhf, gradient) &
            bind(C, name="xtbgb_serverSubmit")
         import :: c_long_long, c_ptr, c_int, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: server
         integer(c_int), value :: natoms
         integer(c_int), intent(in) :: numbers(*)
         real(c_double), intent(in) :: positions(3, *)
         real(c_double), value :: charge
         integer(c_int), value :: uhf
         integer(c_int), value :: gradient
      end function

      integer(c_int) function xtbgb_serverWait(env, server, id, timeout, energy, gradient, charges, info) &
            bind(C, name="xtbgb_serverWait")
         import :: c_int, c_ptr, c_long_long, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: server
         integer(c_long_long), value :: id
         real(c_double), value :: timeout
         real(c_double), intent(out) :: energy
         real(c_double), intent(out), optional :: gradient(3, *)
         real(c_double), intent(out), optional :: charges(*)
         real(c_double), intent(out) :: info(*)
      end function

      subroutine xtbgb_serverStats(env, server, stats) bind(C, name="xtbgb_serverStats")
         import :: c_ptr, c_double
         type(c_ptr), value :: env
         type(c_ptr), value :: server
         real(c_double), intent(out) :: stats(*)
      end subroutine

      subroutine xtbgb_serverInjectAdmissionFailures(env, server, count) &
            bind(C, name="xtbgb_serverInjectAdmissionFailures")
         import :: c_ptr, c_int
         type(c_ptr), value :: env
         type(c_ptr), value :: server
         integer(c_int), value :: count
      end subroutine

      integer(c_int) function xtbgb_repulsionNoAlloc(natoms, numbers, positions, energy, gradient, stream, errbuf, errlen) &
            bind(C, name="xtbgb_repulsionNoAlloc")
         import :: c_int, c_ptr, c_char
         integer(c_int), value :: natoms
         type(c_ptr), value :: numbers
         type(c_ptr), value :: positions
         type(c_ptr), value :: energy
         type(c_ptr), value :: gradient
         type(c_ptr), value :: stream
         character(kind=c_char), intent(out), optional :: errbuf(*)
         integer(c_int), value :: errlen
      end function
   end interface

end module xtb_gb300_api
