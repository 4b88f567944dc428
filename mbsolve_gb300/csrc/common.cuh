// Shared definitions of the mbsolve_gb300 CUDA engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define MBG_HD __host__ __device__ __forceinline__

namespace mbg {

// Physical constants as the reference defines them (types.hpp:36-73).
constexpr double HBAR = 1.05457266e-34;
constexpr double PI = 3.141592653589793238462643383279502884;
constexpr double MU0 = PI * 4e-7;
constexpr double EPS0 = 8.854187817e-12;

// Largest level count served (the reference instantiates 2..6,
// solver-cpu/src/solver_cpu_loader.cpp:41-88).
constexpr int MAX_LEVELS = 6;
constexpr int MAX_V = MAX_LEVELS * MAX_LEVELS - 1;  // 35

// Device status bits (read by the host after a run).
enum : uint32_t {
    STATUS_NONFINITE = 1u,      // a recorded value was NaN or Inf
    STATUS_PRECOMPUTE = 2u,     // the FP64 precompute rejected a material
    STATUS_REGION = 4u,         // a grid point lies in no region
    STATUS_TC_WAIT = 8u,        // a tensor-core or bulk-copy completion wait ran out
    STATUS_PERSIST_WAIT = 16u,  // a persistent-kernel wait for neighbour tiles ran out
};

// Per-tile work item: one contiguous output range of one run.
struct tile_desc {
    uint32_t run;
    int32_t out_start;   // run-local index of the first output cell
    int32_t out_len;     // output cells (<= tile width - 2*halo)
    int32_t uniform_mat; // global material index if every in-run cell of
                         // the tile's input window has it, else -1
};

// Per-run constants of the packed ragged layout.
struct run_desc {
    uint64_t offset;      // global index of the run's cell 0
    uint32_t n_x;
    uint32_t n_t;
    double dx_inv;
    uint32_t src_begin, src_end;
    uint32_t rec_begin, rec_end;
    // mirror boundary (MBG_BC_MIRROR): H beyond the left end = k_left E[0],
    // beyond the right end = -k_right E[n_x - 1]; 0 for PMC (H = 0)
    double k_left, k_right;
};

// A source after set-up (solver_cpu_fdtd.tpp:185-202): grid index and an
// offset into the value tables (n_t values, entry j for time j*dt).
struct src_desc {
    int32_t type;
    uint32_t x_idx;
    uint64_t table_offset;
};

// A record after set-up: copy_list_entry_dev (copy_list_entry.hpp:51-109).
struct rec_desc {
    int32_t type;
    uint32_t row_idx, col_idx;
    uint32_t pos;        // first grid point
    uint32_t cols;
    uint64_t rows;
    double ratio;        // interval ratio dt/interval (1 when every step)
    uint64_t offset;     // into the scratch of the run's records
};

// Schedule of one launch of the persistent time-step kernel (see
// step_kernel_persist): `levels` launches' worth of tiles.
struct persist_params {
    uint32_t levels;     // levels (launches of nsub steps) in this launch
    uint32_t n_tiles;
    uint32_t base;       // levels every tile had finished before this launch
    uint32_t* work;      // work counter, zero at the launch
    uint32_t* prog;      // per tile: levels finished (absolute)
    const int2* nb;      // per tile: left and right neighbour in its run (itself if none)
    uint32_t wait_limit; // polls of a wait for neighbour tiles (0: the kernel's default)
    uint32_t stall;      // 0; tests set 1 << 30 so that every wait runs out
};

// Kernel-side record types beyond MBG_RECORD_*: a coherence record (the
// entry rho[row][col], row != col; the reference records zero) becomes two
// device records, its real and its imaginary part, each stored like a real
// record (the imaginary part rows * cols after the real part).
enum : int32_t { REC_COH_RE = 5, REC_COH_IM = 6 };

// copy_list_entry_dev::hasto_record (copy_list_entry.hpp:269-275). The
// reference evaluates floor(ratio*(0-1)) on an unsigned wrap-around at
// iteration 0, which never equals floor(0): iteration 0 always records.
MBG_HD bool hasto_record(double ratio, uint64_t n)
{
    if (n == 0) return true;
    long long last = (long long) floor(ratio * (double) (n - 1));
    long long next = (long long) floor(ratio * (double) n);
    return last != next;
}

MBG_HD int cvr_len(int N) { return N * N - 1; }

}  // namespace mbg
