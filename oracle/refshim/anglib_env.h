// TEST INFRASTRUCTURE ONLY.  Force-included when the reference's
// new_anglib.C is compiled by itself (oracle/Makefile, target `ref`): that
// file's only use of the reference's global header is the spin-adapted
// switch of its input object, which this stand-in provides (always
// spin-adapted, the only mode this library implements).  The header's own
// include guard is defined on the command line so that nothing else of it
// (Boost, newmat, MPI) is needed.
#pragma once
namespace SpinAdapted {
struct AnglibInput {
  bool spinAdapted() const { return true; }
};
static AnglibInput dmrginp;
}  // namespace SpinAdapted
