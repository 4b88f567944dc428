/*
 * GB300 solver for mbsolve-lib: flattens the reference's device/scenario
 * objects into the C-ABI description and maps the C-ABI's status codes back
 * to the reference's exceptions.
 */
#include <complex>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <typeinfo>
#include <mbsolve/lib.hpp>

#include "solver_gpu_fdtd.hpp"

namespace mbsolve {

namespace {

void check(int rc)
{
    if (rc == MBG_OK) return;
    std::string msg = mbg_last_error();
    if (rc == MBG_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

/* storage the flat description points into, alive during one call */
struct description {
    std::vector<std::vector<double> > arrays;
    std::vector<mbg_qm> qms;
    std::vector<mbg_material> mats;
    std::vector<mbg_region> regions;
    std::vector<mbg_source> sources;
    std::vector<mbg_record> records;
    mbg_device dev;
    mbg_scenario scen;

    const double* keep(std::vector<double> v)
    {
        if (v.empty()) v.push_back(0.0);
        arrays.push_back(std::move(v));
        return arrays.back().data();
    }
};

std::vector<double> packed_off(const qm_operator& op, unsigned int n)
{
    std::vector<double> r;
    for (const auto& c : op.get_off_diagonal()) {
        r.push_back(c.real());
        r.push_back(c.imag());
    }
    r.resize(n, 0.0);
    return r;
}

/* the device part, the scenario's density initial condition and records;
 * sources and sampled fields need the grid and are added afterwards */
void describe(
    std::shared_ptr<const device> dev,
    std::shared_ptr<const scenario> scen,
    description& d)
{
    d.arrays.reserve(64 + 4 * dev->get_used_materials().size());
    const auto& used = dev->get_used_materials(); /* sorted ids */
    d.qms.reserve(used.size());
    std::vector<std::string> ids(used.begin(), used.end());
    for (const auto& id : ids) {
        auto mat = material::get_from_library(id);
        mbg_material m;
        m.rel_permittivity = mat->get_rel_permittivity();
        m.rel_permeability = mat->get_rel_permeability();
        m.overlap_factor = mat->get_overlap_factor();
        m.losses = mat->get_losses();
        m.qm = nullptr;
        auto qm = mat->get_qm();
        if (qm) {
            unsigned int N = qm->get_num_levels();
            mbg_qm q;
            q.num_levels = N;
            q.carrier_density = qm->get_carrier_density();
            q.h_diag = d.keep(qm->get_hamiltonian().get_main_diagonal());
            q.h_off = d.keep(packed_off(qm->get_hamiltonian(), N * (N - 1)));
            q.mu_diag = d.keep(qm->get_dipole_operator().get_main_diagonal());
            q.mu_off = d.keep(packed_off(qm->get_dipole_operator(), N * (N - 1)));
            auto sop = std::dynamic_pointer_cast<qm_lindblad_relaxation>(
                qm->get_relaxation_superop());
            std::vector<double> s(N * N, 0.0), g(N * (N - 1) / 2, 0.0);
            if (sop) {
                q.relax_kind = MBG_RELAX_LINDBLAD;
                const auto& sm = sop->get_scattering_rates();
                for (unsigned int i = 0; i < N; i++)
                    for (unsigned int j = 0; j < N; j++) s[i * N + j] = sm[i][j];
                const auto& dr = sop->get_dephasing_rates();
                for (size_t i = 0; i < g.size() && i < dr.size(); i++) g[i] = dr[i];
            } else if (qm->get_relaxation_superop() &&
                       typeid(*qm->get_relaxation_superop()) != typeid(qm_superop)) {
                throw std::invalid_argument("Unsupported superoperator!");
            } else {
                q.relax_kind = MBG_RELAX_NONE;
            }
            q.scattering = d.keep(s);
            q.dephasing = d.keep(g);
            d.qms.push_back(q);
            m.qm = &d.qms.back();
        }
        d.mats.push_back(m);
    }
    for (const auto& reg : dev->get_regions()) {
        mbg_region r;
        r.material = 0;
        for (size_t i = 0; i < ids.size(); i++)
            if (ids[i] == reg->get_material()->get_id()) r.material = (uint32_t) i;
        r.x_start = reg->get_x_start();
        r.x_end = reg->get_x_end();
        d.regions.push_back(r);
    }
    d.dev.num_materials = (uint32_t) d.mats.size();
    d.dev.materials = d.mats.data();
    d.dev.num_regions = (uint32_t) d.regions.size();
    d.dev.regions = d.regions.data();
    /* the reference's solvers apply H = 0 beyond both ends whatever
     * bc_field the device holds (solver_cpu_fdtd.tpp:263-275) */
    d.dev.bc_kind = MBG_BC_PMC;
    d.dev.refl_left = 1.0;
    d.dev.refl_right = 1.0;

    mbg_scenario& s = d.scen;
    std::memset(&s, 0, sizeof(s));
    s.num_gridpoints = scen->get_num_gridpoints();
    s.endtime = scen->get_endtime();
    s.num_timesteps = scen->get_num_timesteps();
    if (scen->get_ic_density()) {
        /* constant density initial conditions (ic_density_const) */
        qm_operator rho = scen->get_ic_density()->initialize(0.0);
        s.rho_levels = (uint32_t) rho.get_main_diagonal().size();
        s.rho_num_off = (uint32_t) rho.get_off_diagonal().size();
        s.rho_diag = d.keep(rho.get_main_diagonal());
        s.rho_off = d.keep(packed_off(rho, 2 * s.rho_num_off));
    }
    s.e_init_kind = s.h_init_kind = MBG_FIELD_IC_CONST;
    for (const auto& rec : scen->get_records()) {
        mbg_record r;
        r.type = (int32_t) rec->get_type();
        r.row = rec->get_type() == record::density ? rec->get_row() : 0;
        r.col = rec->get_type() == record::density ? rec->get_col() : 0;
        r.interval = rec->get_interval();
        r.position = rec->get_position();
        r.is_complex = rec->is_complex() ? 1 : 0;
        r.coherence = 0; /* off-diagonal entries stay zero, as the reference */
        d.records.push_back(r);
    }
    s.num_records = (uint32_t) d.records.size();
    s.records = d.records.data();
}

/* field initial condition: a constant is passed as such, anything else is
 * sampled at the grid points x = i dx (solver_cpu_fdtd.tpp:127-148) */
void describe_field(
    std::shared_ptr<ic_field> ic,
    const mbg_grid& g,
    description& d,
    int32_t& kind,
    double& value,
    const double*& values)
{
    auto c = std::dynamic_pointer_cast<ic_field_const>(ic);
    if (c) {
        kind = MBG_FIELD_IC_CONST;
        value = c->initialize(0.0);
        return;
    }
    std::vector<double> v(g.num_gridpoints);
    for (uint32_t i = 0; i < g.num_gridpoints; i++) v[i] = ic->initialize(i * g.gridpoint_size);
    kind = MBG_FIELD_IC_VALUES;
    value = 0.0;
    values = d.keep(v);
}

} // namespace

solver_gpu_fdtd::solver_gpu_fdtd(
    const std::string& name,
    std::shared_ptr<const device> dev,
    std::shared_ptr<scenario> scen)
  : solver(name, dev, scen), m_handle(nullptr)
{
    if (dev->get_regions().size() == 0) {
        throw std::invalid_argument("No regions in device!");
    }
    description d;
    describe(dev, scen, d);
    /* the grid first (init_fdtd_simulation, common_fdtd.hpp:52-123) */
    mbg_grid g;
    check(mbg_scenario_grid(&d.dev, &d.scen, &g));
    describe_field(scen->get_ic_electric(), g, d, d.scen.e_init_kind,
                   d.scen.e_init_value, d.scen.e_init_values);
    describe_field(scen->get_ic_magnetic(), g, d, d.scen.h_init_kind,
                   d.scen.h_init_value, d.scen.h_init_values);
    /* sources as value tables get_value(j dt), as the reference precomputes
     * them (solver_cpu_fdtd.tpp:185-202) */
    for (const auto& src : scen->get_sources()) {
        std::vector<double> tab(g.num_timesteps);
        for (uint32_t j = 0; j < g.num_timesteps; j++)
            tab[j] = src->get_value(j * g.timestep_size);
        mbg_source s;
        std::memset(&s, 0, sizeof(s));
        s.type = src->get_type() == source::soft_source ? MBG_SOURCE_SOFT : MBG_SOURCE_HARD;
        s.shape = MBG_SHAPE_TABLE;
        s.position = src->get_position();
        s.table = d.keep(tab);
        s.table_len = g.num_timesteps;
        d.sources.push_back(s);
    }
    d.scen.num_sources = (uint32_t) d.sources.size();
    d.scen.sources = d.sources.data();
    check(mbg_solver_create(name.c_str(), &d.dev, &d.scen, nullptr, &m_handle));
    /* the scenario carries the derived grid, as after init_fdtd_simulation */
    mbg_grid gg;
    check(mbg_solver_grid(m_handle, &gg));
    scen->set_gridpoint_size(gg.gridpoint_size);
    scen->set_timestep_size(gg.timestep_size);
    scen->set_num_timesteps(gg.num_timesteps);
    /* one result per record, in record order (solver_cpu_fdtd.tpp:157-179) */
    uint32_t n = 0;
    check(mbg_solver_num_results(m_handle, &n));
    for (uint32_t k = 0; k < n; k++) {
        uint32_t rows, cols;
        int32_t cplx;
        check(mbg_solver_result_shape(m_handle, k, &rows, &cols, &cplx));
        m_results.push_back(std::make_shared<result>(
            scen->get_records()[k]->get_name(), cols, rows));
    }
}

solver_gpu_fdtd::~solver_gpu_fdtd() { mbg_solver_destroy(m_handle); }

void
solver_gpu_fdtd::run() const
{
    check(mbg_solver_run(m_handle));
    for (size_t k = 0; k < m_results.size(); k++) {
        auto& res = m_results[k];
        std::vector<double> re(res->get_count()), im(res->get_count());
        check(mbg_solver_copy_result(m_handle, (uint32_t) k, re.data(), im.data()));
        std::copy(re.begin(), re.end(), res->get_data_real_it(0, 0));
        std::copy(im.begin(), im.end(), res->get_data_imag_it(0, 0));
    }
}

solver_gpu_loader::solver_gpu_loader()
{
    size_t len = mbg_solver_names(nullptr, 0);
    std::string names(len, '\0');
    mbg_solver_names(&names[0], len);
    std::istringstream in(names.c_str());
    std::string name;
    while (std::getline(in, name)) {
        if (name.empty()) continue;
        solver::register_bootstrap(
            name,
            [name](std::shared_ptr<const device> dev,
                   std::shared_ptr<scenario> scen) {
                return std::make_shared<solver_gpu_fdtd>(name, dev, scen);
            });
    }
}

} // namespace mbsolve
