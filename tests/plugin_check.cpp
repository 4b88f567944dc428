// Checks the mbsolve-lib plugin (mbsolve_gb300/plugin) against the
// reference's own library: registration in the factory, the reference's
// exceptions, the grid written back into the scenario, and, with a GPU,
// one run compared with the reference's init_fdtd_simulation grid.
// Built and run by tests/test_plugin.py.
#include <cmath>
#include <iostream>
#include <mbsolve/lib.hpp>
#include <mbsolve/lib/internal/common_fdtd.hpp>

#include "../mbsolve_gb300/plugin/solver_gpu_fdtd.hpp"

using namespace mbsolve;

static std::shared_ptr<device> make_device(const std::string& tag, bool regions)
{
    auto qm = std::make_shared<qm_desc_2lvl>(1e24, 2 * PI * 2e14, 6.24e-11, 1.0e10, 1.0e10);
    auto vac = std::make_shared<material>("Vacuum" + tag);
    auto ar = std::make_shared<material>("AR_" + tag, qm);
    material::add_to_library(vac);
    material::add_to_library(ar);
    auto dev = std::make_shared<device>("dev" + tag);
    if (regions) {
        dev->add_region(std::make_shared<region>("v1", vac, 0, 7.5e-6));
        dev->add_region(std::make_shared<region>("a", ar, 7.5e-6, 142.5e-6));
        dev->add_region(std::make_shared<region>("v2", vac, 142.5e-6, 150e-6));
    }
    return dev;
}

static std::shared_ptr<scenario> make_scenario()
{
    auto s = std::make_shared<scenario>(
        "Basic", 2048, 100e-15,
        std::make_shared<ic_density_const>(qm_operator({ 1, 0 })),
        std::make_shared<ic_field_const>(0.0));
    s->add_source(std::make_shared<sech_pulse>("sech", 0.0, source::hard_source,
                                               4.2186e9, 2e14, 10, 2e14));
    s->add_record(std::make_shared<record>("inv12", 2.5e-15));
    s->add_record(std::make_shared<record>("e", 0.0, 150e-6));
    return s;
}

int main()
{
    solver_gpu_loader load;
    int n_gpu = 0;
    for (const auto& n : solver::get_avail_solvers())
        if (n.compare(0, 9, "gpu-fdtd-") == 0) n_gpu++;
    std::cout << "registered " << n_gpu << std::endl;

    try {
        solver::create_instance("gpu-fdtd-2lvl-cvr-rodr-fp32", make_device("0", false), make_scenario());
        std::cout << "no-regions: no exception" << std::endl;
    } catch (const std::invalid_argument& e) {
        std::cout << "no-regions: invalid_argument: " << e.what() << std::endl;
    }
    try {
        solver::create_instance("gpu-fdtd-3lvl-cvr-rodr-fp32", make_device("1", true), make_scenario());
        std::cout << "levels: no exception" << std::endl;
    } catch (const std::invalid_argument& e) {
        std::cout << "levels: invalid_argument: " << e.what() << std::endl;
    } catch (const std::exception& e) {
        std::cout << "levels: other: " << e.what() << std::endl;
    }
    try {
        solver::register_bootstrap("gpu-fdtd-noop-fp32", nullptr);
    } catch (const std::invalid_argument& e) {
        std::cout << "duplicate: invalid_argument: " << e.what() << std::endl;
    }

    // grid: the C-ABI's host derivation against the reference's own
    auto dev = make_device("2", true);
    auto ref_scen = make_scenario();
    init_fdtd_simulation(dev, ref_scen, 0.5);
    auto scen = make_scenario();
    try {
        auto sol = solver::create_instance("gpu-fdtd-2lvl-cvr-rodr-fp64", dev, scen);
        bool same = scen->get_num_timesteps() == ref_scen->get_num_timesteps() &&
            scen->get_timestep_size() == ref_scen->get_timestep_size() &&
            scen->get_gridpoint_size() == ref_scen->get_gridpoint_size();
        std::cout << "grid: " << (same ? "same" : "different") << std::endl;
        sol->run();
        const auto& res = sol->get_results();
        double s = 0;
        for (double v : res[1]->get_data_real()) s += v * v;
        std::cout << "run: " << res.size() << " results, rows " << res[1]->get_rows()
                  << ", probe norm " << std::sqrt(s) << std::endl;
    } catch (const std::runtime_error& e) {
        std::cout << "create: runtime_error: " << e.what() << std::endl;
    }
    return 0;
}
