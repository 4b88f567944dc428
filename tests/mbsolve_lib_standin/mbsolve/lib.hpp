/*
 * TEST INFRASTRUCTURE: a stand-in for the part of mbsolve-lib that the
 * GB300 plugin (mbsolve_gb300/plugin/solver_gpu_fdtd.cpp) and its check
 * program use, for machines that have a GPU but not the reference's source
 * tree. Same class, method and enum names and the same meaning as the
 * reference's headers (mbsolve-lib/include/mbsolve/lib/*.hpp, cited per
 * class), written here as plain header-only C++; nothing outside the
 * subset the plugin calls. The plugin is also built against the reference's
 * own library where that tree exists (tests/test_plugin.py).
 */
#ifndef MBSOLVE_LIB_STANDIN_H
#define MBSOLVE_LIB_STANDIN_H

#include <cmath>
#include <complex>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace mbsolve {

/* types.hpp:36-73 */
typedef double real;
const real PI = 3.14159265358979323846264338327950288;
const real HBAR = 1.05457266e-34;
const real E0 = 1.60217733e-19;
const real MU0 = PI * 4e-7;
const real EPS0 = 8.854187817e-12;

/* qm_description.hpp:42-108: Hermitian operator, main diagonal and the
 * upper triangle in column-major order */
class qm_operator
{
    std::vector<real> m_main;
    std::vector<std::complex<real> > m_off;

public:
    explicit qm_operator(
        const std::vector<real>& main_diagonal,
        const std::vector<std::complex<real> >& off_diagonal = {})
      : m_main(main_diagonal), m_off(off_diagonal)
    {}
    unsigned int get_num_levels() const { return (unsigned int) m_main.size(); }
    const std::vector<real>& get_main_diagonal() const { return m_main; }
    const std::vector<std::complex<real> >& get_off_diagonal() const { return m_off; }
};

/* qm_description.hpp:112-164 */
class qm_superop
{
protected:
    unsigned int m_num_levels;

public:
    explicit qm_superop(unsigned int num_levels) : m_num_levels(num_levels) {}
    virtual ~qm_superop() {}
    unsigned int get_num_levels() const { return m_num_levels; }
};

/* qm_description.hpp:166-236: the constructor replaces the diagonal of the
 * scattering matrix by minus the column sums of the off-diagonal rates, and
 * each pair's dephasing rate (upper triangle, column-major) by
 * -|pure| - (|S_mm| + |S_nn|) / 2 with the new diagonal */
class qm_lindblad_relaxation : public qm_superop
{
    std::vector<std::vector<real> > m_scattering;
    std::vector<real> m_dephasing;

public:
    qm_lindblad_relaxation(
        const std::vector<std::vector<real> >& scattering_rates,
        const std::vector<real>& pure_dephasing_rates)
      : qm_superop((unsigned int) scattering_rates.size()),
        m_scattering(scattering_rates), m_dephasing(pure_dephasing_rates)
    {
        const unsigned int n = m_num_levels;
        for (unsigned int m = 0; m < n; m++) {
            real s = 0.0;
            for (unsigned int j = 0; j < n; j++)
                if (j != m) s += m_scattering[j][m];
            m_scattering[m][m] = -s;
        }
        unsigned int q = 0;
        for (unsigned int k = 1; k < n; k++)
            for (unsigned int j = 0; j < k; j++, q++)
                m_dephasing[q] = -std::fabs(m_dephasing[q]) -
                    0.5 * (std::fabs(m_scattering[j][j]) + std::fabs(m_scattering[k][k]));
    }
    const std::vector<std::vector<real> >& get_scattering_rates() const { return m_scattering; }
    const std::vector<real>& get_dephasing_rates() const { return m_dephasing; }
};

/* qm_description.hpp:238-300 */
class qm_description
{
    real m_density;
    qm_operator m_h, m_u;
    std::shared_ptr<qm_superop> m_relax;

public:
    qm_description(
        real carrier_density,
        const qm_operator& hamiltonian,
        const qm_operator& dipole_operator,
        std::shared_ptr<qm_superop> relaxation_superop)
      : m_density(carrier_density), m_h(hamiltonian), m_u(dipole_operator),
        m_relax(relaxation_superop)
    {}
    virtual ~qm_description() {}
    real get_carrier_density() const { return m_density; }
    unsigned int get_num_levels() const { return m_h.get_num_levels(); }
    const qm_operator& get_hamiltonian() const { return m_h; }
    const qm_operator& get_dipole_operator() const { return m_u; }
    std::shared_ptr<qm_superop> get_relaxation_superop() const { return m_relax; }
};

/* qm_description.hpp:338-432: two levels, H = hbar/2 diag(-w0, w0), dipole
 * off-diagonal -E0 d, relaxation towards the equilibrium inversion w */
class qm_desc_2lvl : public qm_description
{
public:
    qm_desc_2lvl(
        real carrier_density,
        real transition_freq,
        real dipole_moment,
        real scattering_rate,
        real dephasing_rate,
        real equilibrium_inversion = -1.0)
      : qm_description(
            carrier_density,
            qm_operator({ -HBAR * transition_freq / 2, HBAR * transition_freq / 2 }),
            qm_operator({ 0.0, 0.0 }, { std::complex<real>(-E0 * dipole_moment, 0.0) }),
            std::make_shared<qm_lindblad_relaxation>(
                std::vector<std::vector<real> >{
                    { 0.0, scattering_rate * 0.5 * (1 - equilibrium_inversion) },
                    { scattering_rate * 0.5 * (1 + equilibrium_inversion), 0.0 } },
                std::vector<real>{ dephasing_rate - 0.5 * scattering_rate }))
    {}
};

/* material.hpp:40-135 */
class material
{
    std::string m_id;
    std::shared_ptr<qm_description> m_qm;
    real m_eps_r, m_overlap, m_losses, m_mu_r;
    static std::map<std::string, std::shared_ptr<material> >& lib()
    {
        static std::map<std::string, std::shared_ptr<material> > l;
        return l;
    }

public:
    explicit material(
        const std::string& id,
        std::shared_ptr<qm_description> qm = nullptr,
        real rel_permittivity = 1.0,
        real overlap_factor = 1.0,
        real losses = 0.0,
        real rel_permeability = 1.0)
      : m_id(id), m_qm(qm), m_eps_r(rel_permittivity), m_overlap(overlap_factor),
        m_losses(losses), m_mu_r(rel_permeability)
    {}
    const std::string& get_id() const { return m_id; }
    std::shared_ptr<qm_description> get_qm() const { return m_qm; }
    real get_rel_permittivity() const { return m_eps_r; }
    real get_rel_permeability() const { return m_mu_r; }
    real get_overlap_factor() const { return m_overlap; }
    real get_losses() const { return m_losses; }
    static void add_to_library(std::shared_ptr<material> m) { lib()[m->get_id()] = m; }
    static std::shared_ptr<material> get_from_library(const std::string& id)
    {
        auto it = lib().find(id);
        if (it == lib().end()) throw std::invalid_argument("Id not found in library.");
        return it->second;
    }
};

/* device.hpp:82-150 */
class region
{
    std::string m_name;
    std::shared_ptr<material> m_mat;
    real m_x0, m_x1;

public:
    region(const std::string& name, std::shared_ptr<material> mat, real x_start, real x_end)
      : m_name(name), m_mat(mat), m_x0(x_start), m_x1(x_end)
    {}
    const std::string& get_name() const { return m_name; }
    std::shared_ptr<material> get_material() const { return m_mat; }
    real get_x_start() const { return m_x0; }
    real get_x_end() const { return m_x1; }
};

/* device.hpp:152-216 */
class device
{
    std::string m_name;
    std::vector<std::shared_ptr<region> > m_regions;
    std::set<std::string> m_used;

public:
    explicit device(const std::string& name) : m_name(name) {}
    void add_region(std::shared_ptr<region> reg)
    {
        m_regions.push_back(reg);
        m_used.insert(reg->get_material()->get_id());
    }
    const std::vector<std::shared_ptr<region> >& get_regions() const { return m_regions; }
    const std::set<std::string>& get_used_materials() const { return m_used; }
};

/* scenario.hpp:40-157 */
class ic_density
{
public:
    virtual ~ic_density() {}
    virtual qm_operator initialize(real x) = 0;
};
class ic_density_const : public ic_density
{
    qm_operator m_rho;

public:
    explicit ic_density_const(const qm_operator& rho) : m_rho(rho) {}
    qm_operator initialize(real) { return m_rho; }
};
class ic_field
{
public:
    virtual ~ic_field() {}
    virtual real initialize(real x) = 0;
};
class ic_field_const : public ic_field
{
    real m_v;

public:
    explicit ic_field_const(real v) : m_v(v) {}
    real initialize(real) { return m_v; }
};

/* source.hpp:35-196 */
class source
{
public:
    enum type { hard_source, soft_source };

protected:
    std::string m_name;
    real m_position;
    type m_type;
    real m_ampl, m_freq, m_phase;

public:
    source(const std::string& name, real position, type source_type, real ampl, real freq, real phase = 0)
      : m_name(name), m_position(position), m_type(source_type), m_ampl(ampl), m_freq(freq),
        m_phase(phase)
    {}
    virtual ~source() {}
    virtual real calc_value(real) const { return 0.0; }
    real get_value(real t, real = 0.0) const { return m_ampl * calc_value(t); }
    real get_position() const { return m_position; }
    type get_type() const { return m_type; }
};
/* A sech(beta t - phase) sin(2 pi f t - phase_sin) */
class sech_pulse : public source
{
    real m_beta, m_phase_sin;

public:
    sech_pulse(
        const std::string& name,
        real position,
        type source_type,
        real ampl,
        real freq,
        real phase,
        real beta,
        real phase_sin = 0.0)
      : source(name, position, source_type, ampl, freq, phase), m_beta(beta), m_phase_sin(phase_sin)
    {}
    real calc_value(real t) const
    {
        return 1.0 / std::cosh(m_beta * t - m_phase) * std::sin(2 * PI * m_freq * t - m_phase_sin);
    }
};

/* record.hpp:37-140: one-based density indices in the constructor, stored
 * zero-based */
class record
{
public:
    enum type { electric, polar_dt, magnetic, density, inversion };

private:
    std::string m_name;
    type m_type;
    unsigned int m_row, m_col;
    real m_interval, m_position;
    bool m_is_complex;

public:
    /* type from the name's first letter (record.cpp:27-56) */
    record(const std::string& name, real interval, real position = -1.0)
      : m_name(name), m_row(0), m_col(0), m_interval(interval), m_position(position)
    {
        switch (name.empty() ? ' ' : name[0]) {
        case 'e': m_type = electric; break;
        case 'h': m_type = magnetic; break;
        case 'p': m_type = polar_dt; break;
        case 'd': m_type = density; break;
        case 'i': m_type = inversion; break;
        default: throw std::invalid_argument("Unknown record type");
        }
        m_is_complex = m_type == density && m_row != m_col;
    }
    record(
        const std::string& name,
        type record_type,
        unsigned int row_idx,
        unsigned int col_idx,
        real interval,
        real position)
      : m_name(name), m_type(record_type), m_row(row_idx - 1), m_col(col_idx - 1),
        m_interval(interval), m_position(position)
    {
        m_is_complex = m_type == density && m_row != m_col;
    }
    std::string get_name() const { return m_name; }
    type get_type() const { return m_type; }
    unsigned int get_row() const { return m_row; }
    unsigned int get_col() const { return m_col; }
    real get_interval() const { return m_interval; }
    real get_position() const { return m_position; }
    bool is_complex() const { return m_is_complex; }
};

/* result.hpp:37-120: row-major rows x cols */
class result
{
    std::string m_name;
    unsigned int m_cols, m_rows;
    std::vector<real> m_real, m_imag;

public:
    result(const std::string& name, unsigned int cols, unsigned int rows, bool = false)
      : m_name(name), m_cols(cols), m_rows(rows), m_real((size_t) cols * rows),
        m_imag((size_t) cols * rows)
    {}
    std::string get_name() const { return m_name; }
    unsigned int get_count() const { return m_cols * m_rows; }
    unsigned int get_cols() const { return m_cols; }
    unsigned int get_rows() const { return m_rows; }
    std::vector<real>::iterator get_data_real_it(unsigned int row, unsigned int col)
    {
        return m_real.begin() + (size_t) row * m_cols + col;
    }
    std::vector<real>::iterator get_data_imag_it(unsigned int row, unsigned int col)
    {
        return m_imag.begin() + (size_t) row * m_cols + col;
    }
    const std::vector<real>& get_data_real() const { return m_real; }
};

/* scenario.hpp:164-335 */
class scenario
{
    std::string m_name;
    unsigned int m_nx, m_nt;
    real m_endtime, m_dt = 0, m_dx = 0;
    std::shared_ptr<ic_density> m_dens;
    std::shared_ptr<ic_field> m_e, m_h;
    std::vector<std::shared_ptr<source> > m_sources;
    std::vector<std::shared_ptr<record> > m_records;

public:
    scenario(
        const std::string& name,
        unsigned int num_gridpoints,
        real endtime,
        std::shared_ptr<ic_density> density_init,
        std::shared_ptr<ic_field> electric_init,
        std::shared_ptr<ic_field> magnetic_init = std::make_shared<ic_field_const>(0.0),
        unsigned int num_timesteps = 2)
      : m_name(name), m_nx(num_gridpoints), m_nt(num_timesteps), m_endtime(endtime),
        m_dens(density_init), m_e(electric_init), m_h(magnetic_init)
    {}
    void add_source(std::shared_ptr<source> s) { m_sources.push_back(s); }
    void add_record(std::shared_ptr<record> r) { m_records.push_back(r); }
    const std::vector<std::shared_ptr<source> >& get_sources() const { return m_sources; }
    const std::vector<std::shared_ptr<record> >& get_records() const { return m_records; }
    unsigned int get_num_gridpoints() const { return m_nx; }
    unsigned int get_num_timesteps() const { return m_nt; }
    real get_endtime() const { return m_endtime; }
    real get_timestep_size() const { return m_dt; }
    real get_gridpoint_size() const { return m_dx; }
    void set_num_timesteps(unsigned int v) { m_nt = v; }
    void set_timestep_size(real v) { m_dt = v; }
    void set_gridpoint_size(real v) { m_dx = v; }
    std::shared_ptr<ic_density> get_ic_density() const { return m_dens; }
    std::shared_ptr<ic_field> get_ic_electric() const { return m_e; }
    std::shared_ptr<ic_field> get_ic_magnetic() const { return m_h; }
};

} // namespace mbsolve

#include <mbsolve/lib/solver.hpp>

#endif
