/*
 * TEST INFRASTRUCTURE: stand-in for mbsolve-lib's solver factory
 * (mbsolve-lib/include/mbsolve/lib/solver.hpp:42-142, src/solver.cpp:26-84)
 * with the same names and behaviour: a name -> bootstrap map, a duplicate
 * name throws std::invalid_argument("Solver already registered."), an
 * unknown one std::invalid_argument("Unknown solver " + name). See
 * tests/mbsolve_lib_standin/mbsolve/lib.hpp.
 */
#ifndef MBSOLVE_LIB_STANDIN_SOLVER_H
#define MBSOLVE_LIB_STANDIN_SOLVER_H

#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace mbsolve {

class device;
class scenario;
class result;

class solver
{
public:
    typedef std::function<std::shared_ptr<solver>(
        std::shared_ptr<const device> dev,
        std::shared_ptr<scenario> scen)>
        bootstrap_t;

private:
    static std::map<std::string, bootstrap_t>& bootstraps()
    {
        static std::map<std::string, bootstrap_t> m;
        return m;
    }

protected:
    solver(const std::string& name, std::shared_ptr<const device> dev, std::shared_ptr<scenario> scen)
      : m_name(name), m_device(dev), m_scenario(scen)
    {}
    std::string m_name;
    std::shared_ptr<const device> m_device;
    std::shared_ptr<scenario> m_scenario;
    std::vector<std::shared_ptr<result> > m_results;

public:
    virtual ~solver() {}
    static std::vector<std::string> get_avail_solvers()
    {
        std::vector<std::string> v;
        for (const auto& kv : bootstraps()) v.push_back(kv.first);
        return v;
    }
    static void register_bootstrap(const std::string& name, bootstrap_t b)
    {
        if (bootstraps().count(name)) throw std::invalid_argument("Solver already registered.");
        bootstraps()[name] = b;
    }
    static std::shared_ptr<solver> create_instance(
        const std::string& name,
        std::shared_ptr<const device> dev,
        std::shared_ptr<scenario> scen)
    {
        auto it = bootstraps().find(name);
        if (it == bootstraps().end()) throw std::invalid_argument("Unknown solver " + name);
        return it->second(dev, scen);
    }
    const std::string& get_name() const { return m_name; }
    virtual void run() const = 0;
    const std::vector<std::shared_ptr<result> >& get_results() const { return m_results; }
};

} // namespace mbsolve

#endif
