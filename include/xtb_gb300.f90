! ISO_C_BINDING interface of libxtb_gb300.so for Fortran hosts.
!
! Binds the C API declared in xtb.h (the same symbols as the reference's
! include/xtb.h:71-310) and the batched extension of xtb_gb300.h.  Handles are
! opaque type(c_ptr); arrays are passed by address in Fortran (column-major)
! order, so positions(3, natoms) and gradient(3, natoms) map directly onto the
! C layout [natoms][3].  Link with -lxtb_gb300.
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
   end interface

end module xtb_gb300_api
