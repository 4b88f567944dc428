/*
 * ORACLE — test infrastructure only.
 *
 * Eigen-free density algorithms with the static interface the reference's
 * time loops expect (solver_cpu_fdtd.tpp / solver_cpu_fdtd_red.tpp:
 * name, density, sim_constants, allocator, get_qm_constants, update,
 * calc_inversion, calc_population, get_density). They let the reference's
 * own, unmodified time loops run here, where Eigen (which the reference's
 * algo_lindblad_cvr_rodr.hpp and algo_lindblad_reg_cayley.hpp include) is
 * not installed. The numerics are the oracle's restatement (mb_oracle.cpp),
 * which this header includes; the interface mirrors
 * mbsolve-lib/include/mbsolve/lib/internal/algo_lindblad_cvr_rodr.hpp:41-300
 * and algo_lindblad_reg_cayley.hpp:44-275.
 */
#ifndef MBSOLVE_GB300_ORACLE_REF_ALGOS_HPP
#define MBSOLVE_GB300_ORACLE_REF_ALGOS_HPP

#include <array>
#include <memory>
#include <mbsolve/lib/qm_description.hpp>

#include "mb_oracle.cpp"

namespace mbsolve {

/* reference qm_description -> oracle description */
inline mbo::qm_desc to_oracle_qm(const qm_description& q)
{
    mbo::qm_desc d;
    d.N = (int) q.get_num_levels();
    d.carrier_density = q.get_carrier_density();
    d.h_diag = q.get_hamiltonian().get_main_diagonal();
    d.h_off = q.get_hamiltonian().get_off_diagonal();
    d.mu_diag = q.get_dipole_operator().get_main_diagonal();
    d.mu_off = q.get_dipole_operator().get_off_diagonal();
    auto sop = std::dynamic_pointer_cast<qm_lindblad_relaxation>(
        q.get_relaxation_superop());
    if (sop) {
        d.relax_kind = MBG_RELAX_LINDBLAD;
        d.scattering = sop->get_scattering_rates();
        d.dephasing = sop->get_dephasing_rates();
    } else {
        d.relax_kind = MBG_RELAX_NONE;
    }
    return d;
}

template<unsigned int num_lvl>
class lindblad_cvr_rodr_ref
{
public:
    static const unsigned int vec_len = num_lvl * num_lvl - 1;
    static std::string name() { return "cvr-rodr"; }
    typedef std::array<real, vec_len> density;
    typedef mbo::rodr_consts sim_constants;
    typedef std::allocator<sim_constants> allocator;

    static sim_constants get_qm_constants(
        std::shared_ptr<const qm_description> qm,
        real time_step)
    {
        if (qm) {
            mbo::qm_desc d = to_oracle_qm(*qm);
            return mbo::rodr_constants(&d, num_lvl, time_step);
        }
        return mbo::rodr_constants(nullptr, num_lvl, time_step);
    }

    static inline void
    update(const sim_constants& sc, density& d, real e, real* p_t)
    {
        mbo::rodr_update(sc, num_lvl, d.data(), e, p_t);
    }

    static inline real calc_inversion(const density& d)
    {
        return d[num_lvl * (num_lvl - 1)];
    }

    static inline real calc_population(const density& d, unsigned int idx)
    {
        return mbo::cvr_population(num_lvl, d.data(), idx);
    }

    static inline density get_density(const qm_operator& op)
    {
        std::vector<real> v = mbo::coherence_vector(
            num_lvl, op.get_main_diagonal(), op.get_off_diagonal());
        density r;
        std::copy(v.begin(), v.end(), r.begin());
        return r;
    }

    static inline density get_density()
    {
        density r;
        r.fill(0.0);
        return r;
    }
};

template<unsigned int num_lvl>
class lindblad_reg_cayley_ref
{
public:
    static std::string name() { return "reg-cayley"; }
    struct density {
        mbo::cmat m;
        density() : m(num_lvl) {}
    };
    typedef mbo::cayley_consts sim_constants;
    typedef std::allocator<sim_constants> allocator;

    static sim_constants get_qm_constants(
        std::shared_ptr<const qm_description> qm,
        real time_step)
    {
        if (qm) {
            mbo::qm_desc d = to_oracle_qm(*qm);
            return mbo::cayley_constants(&d, num_lvl, time_step);
        }
        return mbo::cayley_constants(nullptr, num_lvl, time_step);
    }

    static inline void
    update(const sim_constants& sc, density& d, real e, real* p_t)
    {
        mbo::cayley_update(sc, d.m, e, p_t);
    }

    static inline real calc_inversion(const density& d)
    {
        return (d.m(1, 1) - d.m(0, 0)).real();
    }

    static inline real calc_population(const density& d, unsigned int idx)
    {
        return d.m(idx, idx).real();
    }

    static inline density get_density(const qm_operator& op)
    {
        density r;
        r.m = mbo::op_to_mat(
            num_lvl, op.get_main_diagonal(), op.get_off_diagonal());
        return r;
    }

    static inline density get_density() { return density(); }
};

} // namespace mbsolve

#endif
