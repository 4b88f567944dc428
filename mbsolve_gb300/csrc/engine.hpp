// Host side of the GB300 engine: scenario set-up, device buffers, launch
// plan. Used by the C-ABI in capi.cu.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mbsolve_gb300.h"
#include "common.cuh"
#include "kernels.cuh"
#include "precompute.cuh"

namespace mbg {

struct invalid_argument : std::invalid_argument {
    using std::invalid_argument::invalid_argument;
};
struct cuda_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void check_cuda(cudaError_t e, const char* what);
#define MBG_CK(x) ::mbg::check_cuda((x), #x)

enum algo_t { ALGO_NOOP = 0, ALGO_CVR = 1, ALGO_CAYLEY = 2 };

struct solver_kind {
    algo_t algo;
    int N;      // levels (0 for noop)
    bool fp64;
};

// "gpu-fdtd-{N}lvl-{cvr-rodr|reg-cayley}-{fp32|fp64}", "gpu-fdtd-noop-fp.."
bool parse_solver_name(const std::string& name, solver_kind& k);
std::vector<std::string> solver_names();

// One run after the host part of the reference constructor
// (solver_cpu_fdtd.tpp:36-203).
struct run_setup {
    uint32_t n_x = 0, n_t = 0;
    double dx = 0, dt = 0, endtime = 0;
    std::vector<pre::mat_in> mats;
    struct region_s {
        uint32_t mat;
        double x0, x1;
    };
    std::vector<region_s> regions;
    // MBG_BC_MIRROR: H beyond the left end = k_left E[0], beyond the right
    // end = -k_right E[n_x - 1]; both 0 for the PMC boundary
    double k_left = 0, k_right = 0;
    int e_kind = 0, h_kind = 0;
    double e_val = 0, h_val = 0;
    std::vector<double> e_vals, h_vals;
    struct source_s {
        int type, shape;
        uint32_t x_idx;
        bool on_grid;
        double ampl, freq, phase, beta_or_tau, phase_sin;
        std::vector<double> table;
    };
    std::vector<source_s> sources;
    struct record_s {
        rec_desc d;  // offset relative to the run's first record
        bool is_complex;
        bool coherence = false;  // rho[row][col], row != col (see REC_COH_RE)
    };
    std::vector<record_s> records;
    uint64_t scratch = 0;
};

run_setup setup_run(const solver_kind& k, const mbg_device* dev, const mbg_scenario* scen);

// Launch configuration of the tile kernel.
struct tuning {
    int C = 0, NT = 0, depth = 0, graph = 0;
};

class engine {
public:
    virtual ~engine() {}
    virtual void advance(uint64_t steps) = 0;
    virtual void restart_clock() = 0;  // next step index is 0 again
    virtual uint64_t steps_done() const = 0;
    virtual uint64_t steps_total() const = 0;
    virtual const run_setup& run(uint32_t r) const = 0;
    virtual uint32_t num_runs() const = 0;
    virtual void copy_result(uint32_t run, uint32_t k, double* re, double* im) = 0;
    virtual void copy_probe_rows(uint32_t k, uint64_t row0, uint64_t nrows, double* out) = 0;
    virtual uint64_t cells() const = 0;
    virtual uint32_t tiles() const = 0;
    virtual tuning tuning_used() const = 0;
    virtual int staging() const = 0;  // 0: registers, 1: bulk-copy staging
    virtual int persistent() const = 0;  // 1: one persistent kernel per advance
    virtual void set_timing(bool on) = 0;
    virtual void kernel_time(uint64_t* launches, double* ms, bool reset) = 0;
    virtual uint32_t status() = 0;
    virtual uint64_t launches() const = 0;
    // begin: record a start event; else record a stop event, wait, return ms
    virtual double stream_time(bool begin) = 0;
    // checkpoint of the full time-loop state (fields, density, records,
    // step index) in host memory; load_state refuses a checkpoint of
    // another ensemble shape
    virtual uint64_t state_bytes() const = 0;
    virtual void save_state(void* host, uint64_t bytes) = 0;
    virtual void load_state(const void* host, uint64_t bytes) = 0;
};

std::unique_ptr<engine> make_engine(
    const solver_kind& k,
    std::vector<run_setup>&& runs,
    const mbg_tuning* t);

// FP64 precompute of n materials on the GPU (one thread per material).
void launch_precompute(
    const pre::mat_in* in,
    int n,
    int algo,
    int N,
    double* ws,
    size_t ws_stride,
    double* out,
    int stride,
    int* codes,
    cudaStream_t s);

// Kernel registry: every instantiated (algo, levels, C, NT) launcher.
template<typename T>
using launch_fn = void (*)(const kparams<T>&, unsigned grid, size_t smem, cudaStream_t s);

// the persistent kernel of a launch shape (step_kernel_persist); returns
// the CTAs it runs with (q.levels == 0: only that number, no launch)
template<typename T>
using persist_fn = unsigned (*)(const kparams<T>&, const persist_params&, size_t smem, cudaStream_t s);

template<typename T>
struct kernel_entry {
    int algo, lev, C, NT;
    launch_fn<T> fn;
    int staging;  // 0: tile state loaded into registers, 1: bulk-copy (TMA) staging
    persist_fn<T> pfn;  // null where the shape has no persistent kernel
};

template<typename T>
std::vector<kernel_entry<T> >& kernel_registry();

template<typename T>
bool register_kernel(int algo, int lev, int C, int NT, launch_fn<T> fn, int staging = 0,
                     persist_fn<T> pfn = nullptr);

}  // namespace mbg
