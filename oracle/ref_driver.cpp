/*
 * ORACLE — test infrastructure only.
 *
 * Runs the reference's own, unmodified code on an mbsolve_gb300 scenario
 * description: mbsolve-lib (device, material, scenario, record, source,
 * result, solver factory) and the time loops solver_cpu_fdtd.tpp and
 * solver_cpu_fdtd_red.tpp, instantiated with lindblad_noop (the
 * reference's, compiles without Eigen) and with the Eigen-free algorithms
 * of ref_algos.hpp. Built by oracle/build_ref.sh from the sources where
 * they lie; the output library goes to oracle/_ref/.
 *
 * Solver names registered here are the reference's own
 * (solver-cpu/src/solver_cpu_loader.cpp:32-89).
 */
#include <atomic>
#include <iostream>
#include <cstdio>
#include <map>
#include <mbsolve/lib.hpp>
#include <mbsolve/lib/internal/algo_lindblad_noop.hpp>
#include <mbsolve/solver-cpu/solver_cpu_fdtd.hpp>
#include <mbsolve/solver-cpu/solver_cpu_fdtd.tpp>
#include <mbsolve/solver-cpu/solver_cpu_fdtd_red.hpp>
#include <mbsolve/solver-cpu/solver_cpu_fdtd_red.tpp>

#include "ref_algos.hpp"

namespace {

using namespace mbsolve;

/* per-grid-point initial field values */
class ic_field_values : public ic_field
{
    std::vector<real> m_v;
    std::shared_ptr<scenario>* m_scen;

public:
    ic_field_values(const double* v, size_t n, std::shared_ptr<scenario>* s)
      : m_v(v, v + n), m_scen(s)
    {}
    real initialize(real x)
    {
        size_t i = (size_t) std::llround(x / (*m_scen)->get_gridpoint_size());
        return i < m_v.size() ? m_v[i] : 0.0;
    }
};

/* tabulated source: get_value(j*dt) returns table[j] */
class table_source : public source
{
    std::vector<real> m_t;
    std::shared_ptr<scenario>* m_scen;

public:
    table_source(
        real pos,
        type t,
        const double* v,
        size_t n,
        std::shared_ptr<scenario>* s)
      : source("table", pos, t, 1.0, 0.0), m_t(v, v + n), m_scen(s)
    {}
    real calc_value(real t) const
    {
        size_t j = (size_t) std::llround(t / (*m_scen)->get_timestep_size());
        return j < m_t.size() ? m_t[j] : 0.0;
    }
};

struct loader {
    loader()
    {
        solver::register_solver<solver_cpu_fdtd<0, lindblad_noop> >(
            "cpu-fdtd-noop");
        solver::register_solver<solver_cpu_fdtd_red<0, lindblad_noop> >(
            "cpu-fdtd-red-noop");
#define REG(N)                                                               \
    solver::register_solver<solver_cpu_fdtd<N, lindblad_cvr_rodr_ref> >(    \
        "cpu-fdtd-" #N "lvl-cvr-rodr");                                      \
    solver::register_solver<solver_cpu_fdtd_red<N, lindblad_cvr_rodr_ref> >( \
        "cpu-fdtd-red-" #N "lvl-cvr-rodr");                                  \
    solver::register_solver<solver_cpu_fdtd<N, lindblad_reg_cayley_ref> >(   \
        "cpu-fdtd-" #N "lvl-reg-cayley");                                    \
    solver::register_solver<                                                 \
        solver_cpu_fdtd_red<N, lindblad_reg_cayley_ref> >(                   \
        "cpu-fdtd-red-" #N "lvl-reg-cayley");
        REG(2)
        REG(3)
        REG(4)
        REG(5)
        REG(6)
#undef REG
    }
};

loader* g_loader = nullptr;
std::atomic<int> g_counter(0);
thread_local std::string g_ref_err;

struct handle {
    std::shared_ptr<scenario> scen;
    std::shared_ptr<device> dev;
    std::shared_ptr<solver> sol;
};

qm_operator make_op(
    const double* diag,
    uint32_t N,
    const double* off,
    uint32_t n_off)
{
    std::vector<real> d(diag, diag + N);
    std::vector<std::complex<real> > o;
    for (uint32_t i = 0; i < n_off; i++)
        o.push_back(std::complex<real>(off[2 * i], off[2 * i + 1]));
    return qm_operator(d, o);
}

std::shared_ptr<qm_description> make_qm(const mbg_qm* q)
{
    uint32_t N = q->num_levels;
    std::shared_ptr<qm_superop> relax;
    if (q->relax_kind == MBG_RELAX_LINDBLAD) {
        std::vector<std::vector<real> > s(N, std::vector<real>(N));
        for (uint32_t i = 0; i < N; i++)
            for (uint32_t j = 0; j < N; j++) s[i][j] = q->scattering[i * N + j];
        /* invert the constructor's folding of the lifetime into the
         * dephasing (qm_description.hpp:189-203) */
        std::vector<real> pure;
        unsigned int k = 0;
        for (uint32_t n = 0; n < N; n++)
            for (uint32_t m = 0; m < n; m++) {
                real life = 0.0, lm = 0.0, ln = 0.0;
                for (uint32_t j = 0; j < N; j++) {
                    if (j != m) lm += s[j][m];
                    if (j != n) ln += s[j][n];
                }
                life = 0.5 * (std::fabs(lm) + std::fabs(ln));
                pure.push_back(-(q->dephasing[k] + life));
                k++;
            }
        relax = std::make_shared<qm_lindblad_relaxation>(s, pure);
    } else {
        relax = std::make_shared<qm_superop>(N);
    }
    return std::make_shared<qm_description>(
        q->carrier_density,
        make_op(q->h_diag, N, q->h_off, N * (N - 1) / 2),
        make_op(q->mu_diag, N, q->mu_off, N * (N - 1) / 2),
        relax);
}

} // namespace

extern "C" {

typedef struct mbr_solver mbr_solver;

const char* mbr_last_error(void) { return g_ref_err.c_str(); }

int mbr_create(
    const char* name,
    const mbg_device* d,
    const mbg_scenario* s,
    mbr_solver** out)
{
    try {
        if (!g_loader) g_loader = new loader();
        int id = g_counter++;
        char prefix[32];
        snprintf(prefix, sizeof(prefix), "r%06d_", id);
        handle* h = new handle();
        h->dev = std::make_shared<device>(std::string(prefix) + "dev");
        std::vector<std::shared_ptr<material> > mats;
        for (uint32_t m = 0; m < d->num_materials; m++) {
            const mbg_material& mm = d->materials[m];
            char mid[64];
            snprintf(mid, sizeof(mid), "%sm%04u", prefix, m);
            auto mat = std::make_shared<material>(
                mid,
                mm.qm ? make_qm(mm.qm) : nullptr,
                mm.rel_permittivity,
                mm.overlap_factor,
                mm.losses,
                mm.rel_permeability);
            material::add_to_library(mat);
            mats.push_back(mat);
        }
        for (uint32_t r = 0; r < d->num_regions; r++)
            h->dev->add_region(std::make_shared<region>(
                "region",
                mats[d->regions[r].material],
                d->regions[r].x_start,
                d->regions[r].x_end));
        std::shared_ptr<ic_density> icd;
        if (s->rho_levels)
            icd = std::make_shared<ic_density_const>(
                make_op(s->rho_diag, s->rho_levels, s->rho_off, s->rho_num_off));
        else
            icd = std::make_shared<ic_density_const>(
                qm_operator(std::vector<real>{ 1.0 }));
        std::shared_ptr<ic_field> ice, ich;
        if (s->e_init_kind == MBG_FIELD_IC_VALUES)
            ice = std::make_shared<ic_field_values>(
                s->e_init_values, s->num_gridpoints, &h->scen);
        else
            ice = std::make_shared<ic_field_const>(s->e_init_value);
        if (s->h_init_kind == MBG_FIELD_IC_VALUES)
            ich = std::make_shared<ic_field_values>(
                s->h_init_values, s->num_gridpoints, &h->scen);
        else
            ich = std::make_shared<ic_field_const>(s->h_init_value);
        h->scen = std::make_shared<scenario>(
            "scen",
            s->num_gridpoints,
            s->endtime,
            icd,
            ice,
            ich,
            s->num_timesteps);
        for (uint32_t k = 0; k < s->num_sources; k++) {
            const mbg_source& src = s->sources[k];
            source::type t = src.type == MBG_SOURCE_SOFT ? source::soft_source
                                                         : source::hard_source;
            std::shared_ptr<source> so;
            if (src.shape == MBG_SHAPE_SECH)
                so = std::make_shared<sech_pulse>(
                    "sech",
                    src.position,
                    t,
                    src.ampl,
                    src.freq,
                    src.phase,
                    src.beta_or_tau,
                    src.phase_sin);
            else if (src.shape == MBG_SHAPE_GAUSSIAN)
                so = std::make_shared<gaussian_pulse>(
                    "gauss",
                    src.position,
                    t,
                    src.ampl,
                    src.freq,
                    src.phase,
                    src.beta_or_tau);
            else
                so = std::make_shared<table_source>(
                    src.position, t, src.table, src.table_len, &h->scen);
            h->scen->add_source(so);
        }
        static const record::type types[5] = { record::electric,
                                               record::polar_dt,
                                               record::magnetic,
                                               record::density,
                                               record::inversion };
        for (uint32_t k = 0; k < s->num_records; k++) {
            const mbg_record& r = s->records[k];
            h->scen->add_record(std::make_shared<record>(
                "rec",
                types[r.type],
                r.row + 1,
                r.col + 1,
                r.interval,
                r.position));
        }
        h->sol = solver::create_instance(name, h->dev, h->scen);
        *out = (mbr_solver*) h;
        return MBG_OK;
    } catch (const std::invalid_argument& e) {
        g_ref_err = e.what();
        return MBG_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        g_ref_err = e.what();
        return MBG_ERR_RUNTIME;
    }
}

int mbr_grid(const mbr_solver* hh, mbg_grid* g)
{
    const handle* h = (const handle*) hh;
    g->num_gridpoints = h->scen->get_num_gridpoints();
    g->num_timesteps = h->scen->get_num_timesteps();
    g->gridpoint_size = h->scen->get_gridpoint_size();
    g->timestep_size = h->scen->get_timestep_size();
    g->endtime = h->scen->get_endtime();
    return MBG_OK;
}

int mbr_run(mbr_solver* hh)
{
    try {
        ((handle*) hh)->sol->run();
        return MBG_OK;
    } catch (const std::exception& e) {
        g_ref_err = e.what();
        return MBG_ERR_RUNTIME;
    }
}

int mbr_result_shape(
    const mbr_solver* hh,
    uint32_t k,
    uint32_t* rows,
    uint32_t* cols,
    int32_t* is_complex)
{
    const handle* h = (const handle*) hh;
    const auto& res = h->sol->get_results();
    if (k >= res.size()) {
        g_ref_err = "result index out of range";
        return MBG_ERR_INVALID_ARGUMENT;
    }
    *rows = res[k]->get_rows();
    *cols = res[k]->get_cols();
    *is_complex = res[k]->is_complex();
    return MBG_OK;
}

int mbr_copy_result(const mbr_solver* hh, uint32_t k, double* re, double* im)
{
    const handle* h = (const handle*) hh;
    const auto& res = h->sol->get_results();
    if (k >= res.size()) {
        g_ref_err = "result index out of range";
        return MBG_ERR_INVALID_ARGUMENT;
    }
    const auto& r = res[k]->get_data_real();
    std::copy(r.begin(), r.end(), re);
    if (im) {
        const auto& i = res[k]->get_data_imag();
        std::copy(i.begin(), i.end(), im);
    }
    return MBG_OK;
}

void mbr_destroy(mbr_solver* hh) { delete (handle*) hh; }

} /* extern "C" */
