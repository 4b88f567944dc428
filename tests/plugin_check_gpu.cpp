// Runs the mbsolve-lib plugin (mbsolve_gb300/plugin) through the solver
// factory on the GPU: solver_gpu_loader, solver::create_instance(name, dev,
// scen), run(), get_results(), the way mbsolve-tool does
// (mbsolve-tool.cpp:669-686). Built by tests/test_plugin_gpu.py against the
// reference's mbsolve-lib where that tree exists, else against the stand-in
// headers in tests/mbsolve_lib_standin (same names, same meaning).
//
//   plugin_check_gpu sit SOLVER OUTDIR n_x t_end length ampl beta
//   plugin_check_gpu zio SOLVER OUTDIR
//
// sit: the 2-level medium filling the device with a hard sech source at
// x = 0 and an E probe at the output facet (the parameters of the Python
// preset, passed in); zio: the Ziolkowski self-induced-transparency preset
// (mbsolve-tool.cpp:249-308) on 1,024 points over 60 fs. Writes every
// result's real part to OUTDIR/result<k>.bin (row-major doubles) and prints
// "result k rows cols" and the grid.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <mbsolve/lib.hpp>

#include "../mbsolve_gb300/plugin/solver_gpu_fdtd.hpp"

using namespace mbsolve;

static void sit(
    unsigned int n_x,
    real t_end,
    real length,
    real ampl,
    real beta,
    std::shared_ptr<device>& dev,
    std::shared_ptr<scenario>& scen)
{
    auto qm = std::make_shared<qm_desc_2lvl>(1e24, 2 * PI * 2e14, 1e-29 / E0, 1e9, 1e9, -1.0);
    auto ar = std::make_shared<material>("AR_sit", qm);
    material::add_to_library(ar);
    dev = std::make_shared<device>("sit-2lvl");
    dev->add_region(std::make_shared<region>("Active region", ar, 0.0, length));
    scen = std::make_shared<scenario>(
        "sit", n_x, t_end, std::make_shared<ic_density_const>(qm_operator({ 1, 0 })),
        std::make_shared<ic_field_const>(0.0), std::make_shared<ic_field_const>(0.0));
    scen->add_source(std::make_shared<sech_pulse>("sech", 0.0, source::hard_source, ampl, 2e14, 15.0, beta));
    scen->add_record(std::make_shared<record>("e", 0.0, length));
}

static void zio(std::shared_ptr<device>& dev, std::shared_ptr<scenario>& scen)
{
    auto qm = std::make_shared<qm_desc_2lvl>(1e24, 2 * PI * 2e14, 6.24e-11, 1.0e10, 1.0e10);
    auto vac = std::make_shared<material>("Vacuum");
    auto ar = std::make_shared<material>("AR_Ziolkowski", qm);
    material::add_to_library(vac);
    material::add_to_library(ar);
    dev = std::make_shared<device>("Ziolkowski");
    dev->add_region(std::make_shared<region>("Vacuum left", vac, 0, 7.5e-6));
    dev->add_region(std::make_shared<region>("Active region", ar, 7.5e-6, 142.5e-6));
    dev->add_region(std::make_shared<region>("Vacuum right", vac, 142.5e-6, 150e-6));
    scen = std::make_shared<scenario>(
        "Basic", 1024, 60e-15, std::make_shared<ic_density_const>(qm_operator({ 1, 0, 0 })),
        std::make_shared<ic_field_const>(0.0));
    scen->add_source(std::make_shared<sech_pulse>("sech", 0.0, source::hard_source, 4.2186e9, 2e14, 10, 2e14));
    scen->add_record(std::make_shared<record>("inv12", 2.5e-15));
    scen->add_record(std::make_shared<record>("e", 2.5e-15));
}

int main(int argc, char** argv)
{
    if (argc < 4) {
        std::cerr << "usage: plugin_check_gpu sit|zio SOLVER OUTDIR [...]" << std::endl;
        return 2;
    }
    const std::string mode = argv[1], name = argv[2], out = argv[3];
    std::shared_ptr<device> dev;
    std::shared_ptr<scenario> scen;
    if (mode == "sit" && argc == 9) {
        sit((unsigned int) std::atoi(argv[4]), std::atof(argv[5]), std::atof(argv[6]), std::atof(argv[7]),
            std::atof(argv[8]), dev, scen);
    } else if (mode == "zio") {
        zio(dev, scen);
    } else {
        std::cerr << "bad arguments" << std::endl;
        return 2;
    }
    solver_gpu_loader load;
    try {
        auto sol = solver::create_instance(name, dev, scen);
        std::cout << "grid " << scen->get_num_timesteps() << " " << scen->get_timestep_size() << " "
                  << scen->get_gridpoint_size() << std::endl;
        sol->run();
        const auto& res = sol->get_results();
        for (size_t k = 0; k < res.size(); k++) {
            const auto& r = res[k];
            std::ofstream f(out + "/result" + std::to_string(k) + ".bin", std::ios::binary);
            f.write(reinterpret_cast<const char*>(r->get_data_real().data()),
                    (std::streamsize) (r->get_data_real().size() * sizeof(real)));
            std::cout << "result " << k << " " << r->get_rows() << " " << r->get_cols() << std::endl;
        }
    } catch (const std::invalid_argument& e) {
        std::cout << "invalid_argument: " << e.what() << std::endl;
        return 1;
    } catch (const std::runtime_error& e) {
        std::cout << "runtime_error: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}
