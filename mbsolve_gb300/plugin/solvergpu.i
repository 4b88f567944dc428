/* SWIG module registering the GB300 solvers on import, as solvercpu.i does
 * for the CPU solvers (solver-cpu/swig/solvercpu.i:1-26). Build next to the
 * reference's mbsolve.lib module; link libmbsolve_gb300.so. */
%module solvergpu
%{
#include "solver_gpu_fdtd.hpp"
%}

%init
%{
    mbsolve::solver_gpu_loader gpu_load;
%}

%import(module="mbsolve.lib") "mbsolve/lib.hpp"

%include "exception.i"
%include "std_except.i"
%include "std_string.i"

%exception {
  try {
    $action
  } catch (const std::exception& e) {
    SWIG_exception(SWIG_RuntimeError, e.what());
  }
}
