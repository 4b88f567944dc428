/*
 * GB300 solver for mbsolve-lib.
 *
 * A subclass of mbsolve::solver (mbsolve-lib/include/mbsolve/lib/solver.hpp:
 * 42-142) that runs the time loop of solver_cpu_fdtd (solver-cpu/include/
 * mbsolve/solver-cpu/solver_cpu_fdtd.tpp) on the GPU through the C-ABI of
 * include/mbsolve_gb300.h. Construct it through the factory after creating
 * a solver_gpu_loader (as solver_cpu_loader registers the CPU solvers):
 *
 *     mbsolve::solver_gpu_loader gpu_load;
 *     auto sol = mbsolve::solver::create_instance(
 *         "gpu-fdtd-2lvl-cvr-rodr-fp32", dev, scen);
 *     sol->run();
 *     sol->get_results();
 *
 * Errors: std::invalid_argument for configuration errors (with the
 * reference's messages), std::runtime_error("CUDA: ...") for device errors.
 */
#ifndef MBSOLVE_SOLVER_GPU_FDTD_H
#define MBSOLVE_SOLVER_GPU_FDTD_H

#include <memory>
#include <string>
#include <vector>
#include <mbsolve/lib/solver.hpp>

#include "../../include/mbsolve_gb300.h"

namespace mbsolve {

class solver_gpu_fdtd : public solver
{
public:
    solver_gpu_fdtd(
        const std::string& name,
        std::shared_ptr<const device> dev,
        std::shared_ptr<scenario> scen);

    ~solver_gpu_fdtd();

    void run() const;

private:
    mbg_solver* m_handle;
};

/* Registers every solver name of the C-ABI library in the factory
 * (pattern of solver-cpu/src/solver_cpu_loader.cpp:32-89). */
class solver_gpu_loader
{
public:
    solver_gpu_loader();
};

} // namespace mbsolve

#endif
