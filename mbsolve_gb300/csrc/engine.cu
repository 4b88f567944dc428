// Host engine: the reference constructor's set-up (solver_cpu_fdtd.tpp:
// 36-203) for one or many runs, the packed ragged layout in HBM, the FP64
// precompute on the GPU, the tile plan, launch loop, CUDA graphs and the
// autotuner.
#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>

#include "engine.hpp"

namespace mbg {

void check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        std::string msg = std::string("CUDA: ") + what + ": " + cudaGetErrorString(e);
        (void) cudaGetLastError();
        throw cuda_error(msg);
    }
}

// ------------------------------------------------------------ registry

template<typename T>
std::vector<kernel_entry<T> >& kernel_registry()
{
    static std::vector<kernel_entry<T> > r;
    return r;
}

template<typename T>
bool register_kernel(int algo, int lev, int C, int NT, launch_fn<T> fn, int staging, persist_fn<T> pfn)
{
    kernel_registry<T>().push_back(kernel_entry<T>{ algo, lev, C, NT, fn, staging, pfn });
    return true;
}

template std::vector<kernel_entry<float> >& kernel_registry<float>();
template std::vector<kernel_entry<double> >& kernel_registry<double>();
template bool register_kernel<float>(int, int, int, int, launch_fn<float>, int, persist_fn<float>);
template bool register_kernel<double>(int, int, int, int, launch_fn<double>, int, persist_fn<double>);

// -------------------------------------------------------------- names

bool parse_solver_name(const std::string& name, solver_kind& k)
{
    const std::string pre = "gpu-fdtd-";
    if (name.compare(0, pre.size(), pre) != 0) return false;
    std::string rest = name.substr(pre.size());
    bool fp64;
    if (rest.size() > 5 && rest.compare(rest.size() - 5, 5, "-fp64") == 0)
        fp64 = true;
    else if (rest.size() > 5 && rest.compare(rest.size() - 5, 5, "-fp32") == 0)
        fp64 = false;
    else
        return false;
    rest = rest.substr(0, rest.size() - 5);
    k.fp64 = fp64;
    if (rest == "noop") {
        k.algo = ALGO_NOOP;
        k.N = 0;
        return true;
    }
    if (rest.size() < 5 || rest[0] < '2' || rest[0] > '6' || rest.compare(1, 4, "lvl-") != 0)
        return false;
    k.N = rest[0] - '0';
    std::string a = rest.substr(5);
    if (a == "cvr-rodr")
        k.algo = ALGO_CVR;
    else if (a == "reg-cayley")
        k.algo = ALGO_CAYLEY;
    else
        return false;
    return true;
}

std::vector<std::string> solver_names()
{
    std::vector<std::string> v;
    for (const char* p : { "fp32", "fp64" }) {
        v.push_back(std::string("gpu-fdtd-noop-") + p);
        for (int n = 2; n <= 6; n++)
            for (const char* a : { "cvr-rodr", "reg-cayley" })
                v.push_back("gpu-fdtd-" + std::to_string(n) + "lvl-" + a + "-" + p);
    }
    return v;
}

// ---------------------------------------------------------- host set-up

static void fill_operator(
    const double* diag,
    const double* off,
    int N,
    double* re,
    double* im)
{
    for (int i = 0; i < N * N; i++) re[i] = im[i] = 0.0;
    for (int i = 0; i < N; i++) re[i * N + i] = diag[i];
    // qm_operator packing: upper triangle column-major
    // (coherence_vector_representation.hpp:99-130)
    for (int k = 1; k < N; k++)
        for (int j = 0; j < k; j++) {
            int q = pre::upper_index(j, k);
            re[j * N + k] = off[2 * q];
            im[j * N + k] = off[2 * q + 1];
            re[k * N + j] = off[2 * q];
            im[k * N + j] = -off[2 * q + 1];
        }
}

run_setup setup_run(const solver_kind& k, const mbg_device* dev, const mbg_scenario* sc)
{
    run_setup r;
    if (!dev || !sc) throw invalid_argument("null device or scenario");
    if (dev->num_regions == 0) throw invalid_argument("No regions in device!");
    // init_fdtd_simulation(dev, scen, 0.5) (common_fdtd.hpp:52-123)
    if (sc->num_gridpoints == 0) throw invalid_argument("Invalid scenario.");
    double min_eps = 1e42, length = 0.0;
    for (uint32_t i = 0; i < dev->num_regions; i++) {
        const mbg_region& rg = dev->regions[i];
        if (rg.material >= dev->num_materials)
            throw invalid_argument("region refers to an unknown material");
        double e = dev->materials[rg.material].rel_permittivity;
        if (e < min_eps) min_eps = e;
        length += rg.x_end - rg.x_start;
    }
    const double courant = 0.5;
    double velocity = 1.0 / std::sqrt(MU0 * EPS0 * min_eps);
    r.n_x = sc->num_gridpoints;
    if (r.n_x == 1) {
        r.dx = 1e13;
        r.n_t = sc->num_timesteps;
        if (r.n_t < 2) throw invalid_argument("Invalid scenario.");
    } else {
        r.dx = length / (r.n_x - 1);
        double d_t = courant * r.dx / velocity;
        r.n_t = (unsigned int) (std::ceil(sc->endtime / d_t) + 1);
    }
    if (sc->endtime > std::numeric_limits<double>::min()) {
        r.dt = sc->endtime / (r.n_t - 1);
    } else {
        r.n_t = 1;
        r.dt = 3.154e10;
    }
    r.endtime = sc->endtime;

    // materials (solver_cpu_fdtd.tpp:76-89)
    for (uint32_t m = 0; m < dev->num_materials; m++) {
        const mbg_material& mt = dev->materials[m];
        pre::mat_in in;
        std::memset(&in, 0, sizeof(in));
        in.eps_r = mt.rel_permittivity;
        in.mu_r = mt.rel_permeability;
        in.overlap = mt.overlap_factor;
        in.losses = mt.losses;
        in.dt = r.dt;
        in.dx = r.dx;
        if (mt.qm && k.algo != ALGO_NOOP) {
            const mbg_qm& q = *mt.qm;
            if ((int) q.num_levels != k.N)
                throw invalid_argument(
                    "Number of energy levels does not match selected solver!");
            int N = k.N;
            in.N = N;
            in.relax_kind = q.relax_kind;
            in.carrier_density = q.carrier_density;
            fill_operator(q.h_diag, q.h_off, N, in.h_re, in.h_im);
            fill_operator(q.mu_diag, q.mu_off, N, in.mu_re, in.mu_im);
            if (q.relax_kind == MBG_RELAX_LINDBLAD) {
                for (int i = 0; i < N * N; i++) in.S[i] = q.scattering[i];
                for (int i = 0; i < N * (N - 1) / 2; i++) in.deph[i] = q.dephasing[i];
            } else if (k.algo == ALGO_CAYLEY) {
                throw invalid_argument("Unsupported superoperator!");
            }
            uint32_t rn = sc->rho_levels;
            if (rn > (uint32_t) MAX_LEVELS) throw invalid_argument("initial density matrix too large");
            in.rho_levels = (int32_t) rn;
            for (uint32_t i = 0; i < rn; i++) in.rho_diag[i] = sc->rho_diag[i];
            // keep the first entries; the last entry always lands in the
            // last kept slot (the coherence vector keeps only that one)
            uint32_t no = sc->rho_num_off, kept = no < 15 ? no : 15;
            in.rho_num_off = (int32_t) kept;
            for (uint32_t i = 0; i < kept; i++) {
                uint32_t src = (i + 1 == kept) ? no - 1 : i;
                in.rho_off_re[i] = sc->rho_off[2 * src];
                in.rho_off_im[i] = sc->rho_off[2 * src + 1];
            }
        }
        r.mats.push_back(in);
    }
    for (uint32_t i = 0; i < dev->num_regions; i++)
        r.regions.push_back({ dev->regions[i].material, dev->regions[i].x_start,
                              dev->regions[i].x_end });
    // field boundary: the reference applies H = 0 beyond both ends whatever
    // bc_field it is given (solver_cpu_fdtd.tpp:263-275); MBG_BC_MIRROR ties
    // H beyond each end to the end point's E (impedance wall of reflection
    // coefficient r = sqrt(refl) for E)
    if (dev->bc_kind == MBG_BC_MIRROR) {
        if (!(dev->refl_left >= 0.0 && dev->refl_left <= 1.0 && dev->refl_right >= 0.0 &&
              dev->refl_right <= 1.0))
            throw invalid_argument("mirror reflectivity must lie in [0, 1]");
        auto wall = [&](double x, double refl) {
            // material of the end point: the first region containing it
            // (solver_cpu_fdtd.tpp:119-125)
            const mbg_material* mt = nullptr;
            for (uint32_t i = 0; i < dev->num_regions && !mt; i++)
                if (x >= dev->regions[i].x_start && x <= dev->regions[i].x_end)
                    mt = &dev->materials[dev->regions[i].material];
            if (!mt) throw invalid_argument("region not found");
            const double z = std::sqrt(MU0 * mt->rel_permeability / (EPS0 * mt->rel_permittivity));
            const double rr = std::sqrt(refl);
            return (1.0 - rr) / ((1.0 + rr) * z);
        };
        if (r.n_x > 1) {
            r.k_left = wall(0.0, dev->refl_left);
            r.k_right = wall((r.n_x - 1) * r.dx, dev->refl_right);
        }
    } else if (dev->bc_kind != MBG_BC_PMC) {
        throw invalid_argument("unknown field boundary condition");
    }
    // initial fields
    r.e_kind = sc->e_init_kind;
    r.e_val = sc->e_init_value;
    r.h_kind = sc->h_init_kind;
    r.h_val = sc->h_init_value;
    if (r.e_kind == MBG_FIELD_IC_VALUES) {
        if (!sc->e_init_values) throw invalid_argument("missing E initial values");
        r.e_vals.assign(sc->e_init_values, sc->e_init_values + r.n_x);
    }
    if (r.h_kind == MBG_FIELD_IC_VALUES) {
        if (!sc->h_init_values) throw invalid_argument("missing H initial values");
        r.h_vals.assign(sc->h_init_values, sc->h_init_values + r.n_x);
    }
    // records (solver_cpu_fdtd.tpp:157-182, copy_list_entry.hpp:127-171)
    uint64_t scratch = 0;
    for (uint32_t i = 0; i < sc->num_records; i++) {
        const mbg_record& rc = sc->records[i];
        run_setup::record_s rs;
        rec_desc& d = rs.d;
        if (rc.type < 0 || rc.type > 4) throw invalid_argument("Unknown record type");
        d.type = rc.type;
        d.row_idx = rc.row;
        d.col_idx = rc.col;
        // coherence records (no reference counterpart) need a density
        // matrix entry that exists; otherwise they stay zero like the
        // reference's
        rs.coherence = rc.coherence && rc.type == MBG_RECORD_DENSITY && rc.row != rc.col &&
            rc.is_complex && k.algo != ALGO_NOOP && (int) rc.row < k.N && (int) rc.col < k.N;
        if (rc.interval <= r.dt) {
            d.rows = r.n_t;
            d.ratio = 1.0;
        } else {
            d.rows = (uint64_t) (std::floor(r.endtime / rc.interval) + 1);
            d.ratio = r.dt / rc.interval;
        }
        if (rc.position < 0.0) {
            d.pos = 0;
            d.cols = r.n_x;
        } else {
            double idx = std::round(rc.position / r.dx);
            if (idx >= (double) r.n_x)
                throw invalid_argument("record position outside the device");
            d.pos = (uint32_t) idx;
            d.cols = 1;
        }
        d.offset = scratch;
        rs.is_complex = rc.is_complex != 0;
        scratch += (uint64_t) d.cols * d.rows * (rs.is_complex ? 2 : 1);
        r.records.push_back(rs);
    }
    r.scratch = scratch;
    // sources (solver_cpu_fdtd.tpp:185-202)
    for (uint32_t i = 0; i < sc->num_sources; i++) {
        const mbg_source& s = sc->sources[i];
        run_setup::source_s ss;
        ss.type = s.type;
        ss.shape = s.shape;
        double xi = s.position / r.dx;
        ss.x_idx = (xi >= 0 && xi < 4294967296.0) ? (uint32_t) xi : 0xffffffffu;
        ss.on_grid = ss.x_idx < r.n_x;
        ss.ampl = s.ampl;
        ss.freq = s.freq;
        ss.phase = s.phase;
        ss.beta_or_tau = s.beta_or_tau;
        ss.phase_sin = s.phase_sin;
        if (s.shape == MBG_SHAPE_TABLE) {
            if (!s.table || s.table_len < r.n_t)
                throw invalid_argument("source table shorter than the number of time steps");
            ss.table.assign(s.table, s.table + r.n_t);
        } else if (s.shape != MBG_SHAPE_SECH && s.shape != MBG_SHAPE_GAUSSIAN) {
            throw invalid_argument("unknown source shape");
        }
        r.sources.push_back(ss);
    }
    return r;
}

// ------------------------------------------------------- set-up kernels

__global__ void precompute_kernel(
    const pre::mat_in* in,
    int n,
    int algo,
    int N,
    double* ws,
    size_t ws_stride,
    double* out,
    int stride,
    int* codes)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int rc = 0;
    if (algo == ALGO_CVR)
        rc = pre::cvr_precompute(in[i], N, ws + (size_t) i * ws_stride, out + (size_t) i * stride);
    else if (algo == ALGO_CAYLEY)
        rc = pre::cay_precompute(in[i], N, ws + (size_t) i * ws_stride, out + (size_t) i * stride);
    else
        rc = pre::noop_precompute(in[i], out + (size_t) i * stride);
    codes[i] = rc;
}

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
    cudaStream_t s)
{
    precompute_kernel<<<(unsigned) ((n + 63) / 64), 64, 0, s>>>(in, n, algo, N, ws, ws_stride, out, stride, codes);
}

template<typename T>
__global__ void cast_kernel(const double* in, T* out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x)
        out[i] = (T) in[i];
}

struct init_desc {
    uint64_t offset;
    uint32_t n_x;
    double dx;
    uint32_t reg_begin, reg_end;
    uint32_t mat_base;
    int e_kind, h_kind;
    double e_val, h_val;
    uint64_t e_off, h_off;  // into the FP64 initial-value arrays
};
struct region_dev {
    uint32_t mat;
    double x0, x1;
};

// Material map (first region with x_start <= x <= x_end, x = i dx;
// solver_cpu_fdtd.tpp:113-125) and initial state (:127-154).
template<typename T>
__global__ void init_kernel(
    const init_desc* runs,
    uint32_t n_runs,
    const region_dev* regs,
    const double* e_vals,
    const double* h_vals,
    const double* mc64,
    int mstride,
    int algo,
    int N,
    int planes,
    int32_t* mat,
    T* E,
    T* H,
    T* P,
    T* D,
    T* El,  // low parts of the double-float fields (FP32), or null
    T* Hl,
    uint64_t plane,
    uint32_t* status)
{
    for (uint32_t r = blockIdx.y; r < n_runs; r += gridDim.y) {
        const init_desc d = runs[r];
        for (uint64_t l = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; l < d.n_x;
             l += (uint64_t) gridDim.x * blockDim.x) {
            const uint64_t g = d.offset + l;
            const double x = (double) l * d.dx;
            int m = -1;
            for (uint32_t k = d.reg_begin; k < d.reg_end; k++)
                if (x >= regs[k].x0 && x <= regs[k].x1) {
                    m = (int) (d.mat_base + regs[k].mat);
                    break;
                }
            if (m < 0) atomicOr(status, STATUS_REGION);
            mat[g] = m;
            const double e0 = d.e_kind == MBG_FIELD_IC_VALUES ? e_vals[d.e_off + l] : d.e_val;
            const double h0 = d.h_kind == MBG_FIELD_IC_VALUES ? h_vals[d.h_off + l] : d.h_val;
            E[g] = (T) e0;
            H[g] = (T) h0;
            if (El) El[g] = (T) (e0 - (double) E[g]);
            if (Hl) Hl[g] = (T) (h0 - (double) H[g]);
            P[g] = T(0);
            if (m < 0 || planes == 0) continue;
            const double* cb = mc64 + (size_t) m * mstride;
            const bool qm = cb[4] != 0.0;
            if (algo == ALGO_CVR) {
                const pre::cvr_layout L = pre::make_cvr_layout(N);
                const int V = L.V;
                for (int v = 0; v < V; v++) {
                    const double u0 = qm ? cb[L.z0 + v] : 0.0;
                    D[(uint64_t) v * plane + g] = (T) u0;
                    // FP32: the low word of the float pair
                    if (planes == 2 * V) D[(uint64_t) (V + v) * plane + g] = (T) (u0 - (double) (T) u0);
                }
            } else {
                const pre::cay_layout L = pre::make_cay_layout(N);
                const int NN = N * N;
                for (int v = 0; v < NN; v++) {
                    const double r0 = qm ? cb[L.rho0 + v] : 0.0;
                    D[(uint64_t) v * plane + g] = (T) r0;
                    // FP32: the low word of the float pair
                    if (planes == 2 * NN) D[(uint64_t) (NN + v) * plane + g] = (T) (r0 - (double) (T) r0);
                }
            }
        }
    }
}

struct srcgen_desc {
    int shape;
    uint32_t n_t;
    double dt, ampl, freq, phase, beta_or_tau, phase_sin;
    uint64_t table_offset;
};

// Source values get_value(j dt) (source.hpp:94-106, 190-194, 256-260),
// kept in FP64 for both precisions.
__global__ void source_kernel(const srcgen_desc* s, uint32_t n, double* tab)
{
    for (uint32_t k = blockIdx.y; k < n; k += gridDim.y) {
        const srcgen_desc d = s[k];
        for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < d.n_t;
             j += (uint64_t) gridDim.x * blockDim.x) {
            const double t = (double) j * d.dt;
            double v;
            if (d.shape == MBG_SHAPE_SECH)
                v = d.ampl * (1 / cosh(d.beta_or_tau * t - d.phase) * sin(2 * PI * d.freq * t - d.phase_sin));
            else
                v = d.ampl *
                    (exp(-(t - d.phase) * (t - d.phase) / (d.beta_or_tau * d.beta_or_tau)) *
                     sin(2 * PI * d.freq * t));
            tab[d.table_offset + j] = v;
        }
    }
}

// uniform_mat of each tile: the material shared by every in-run point of
// the tile's input window, or -1
__global__ void tile_uniform_kernel(
    tile_desc* tiles,
    uint32_t n_tiles,
    const run_desc* runs,
    const int32_t* mat,
    int halo)
{
    const uint32_t t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (t >= n_tiles) return;
    const tile_desc td = tiles[t];
    const run_desc rd = runs[td.run];
    const int64_t lo = max((int64_t) 0, (int64_t) td.out_start - halo);
    const int64_t hi = min((int64_t) rd.n_x, (int64_t) td.out_start + td.out_len + halo);
    const int32_t m0 = mat[rd.offset + lo];
    bool same = true;
    for (int64_t l = lo + lane; l < hi; l += 32)
        if (mat[rd.offset + l] != m0) same = false;
    // a mirror wall in the window (point 0 or the point beyond the end):
    // the tile takes the non-uniform path, which alone applies the walls
    const int64_t w0 = (int64_t) td.out_start - halo, w1 = (int64_t) td.out_start + td.out_len + halo;
    if ((rd.k_left != 0.0 && w0 <= 0 && 0 < w1) || (rd.k_right != 0.0 && w0 <= (int64_t) rd.n_x && (int64_t) rd.n_x < w1))
        same = false;
    same = __all_sync(0xffffffffu, same);
    if (lane == 0) tiles[t].uniform_mat = same ? m0 : -1;
}

__global__ void step_bump_kernel(unsigned long long* step, unsigned long long add)
{
    *step += add;
}

__global__ void step_set_kernel(unsigned long long* step, unsigned long long v)
{
    *step = v;
}

template<typename T>
__global__ void gather_probe_kernel(
    const T* scratch,
    const uint64_t* offsets,
    uint32_t n_runs,
    uint64_t row0,
    uint64_t nrows,
    T* out)
{
    const uint64_t total = (uint64_t) n_runs * nrows;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < total;
         i += (uint64_t) gridDim.x * blockDim.x) {
        const uint64_t r = i / nrows, k = i % nrows;
        out[i] = scratch[offsets[r] + row0 + k];
    }
}

// --------------------------------------------------------------- engine

template<typename T>
struct dbuf {
    T* p = nullptr;
    size_t n = 0;
    void alloc(size_t count)
    {
        free();
        n = count;
        if (count) MBG_CK(cudaMalloc((void**) &p, count * sizeof(T)));
    }
    void free()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~dbuf() { free(); }
};

static const uint64_t GUARD_FRONT = 512;  // >= largest halo
static const uint64_t GUARD_BACK = 8192;  // >= widest tile
static const int MAX_DEPTH = 256;

static std::mutex g_tune_mutex;
static std::map<std::string, tuning> g_tune_cache;
static bool g_tune_file_read = false;

// Autotuner results persist across processes in the file named by the
// environment variable MBG_TUNE_CACHE, when it is set: one line
// "key C NT depth graph" per tuned problem (keys contain the GPU's name).
// Called with g_tune_mutex held.
static void tune_file_read()
{
    if (g_tune_file_read) return;
    g_tune_file_read = true;
    const char* path = std::getenv("MBG_TUNE_CACHE");
    if (!path || !path[0]) return;
    std::ifstream f(path);
    std::string key;
    tuning t;
    while (f >> key >> t.C >> t.NT >> t.depth >> t.graph)
        if (t.C > 0 && t.NT > 0 && t.depth > 0) g_tune_cache[key] = t;
}

static void tune_file_append(const std::string& key, const tuning& t)
{
    const char* path = std::getenv("MBG_TUNE_CACHE");
    if (!path || !path[0]) return;
    std::ofstream f(path, std::ios::app);
    if (f) f << key << " " << t.C << " " << t.NT << " " << t.depth << " " << t.graph << "\n";
}

template<typename T>
class engine_t : public engine {
public:
    engine_t(const solver_kind& k, std::vector<run_setup>&& runs, const mbg_tuning* t)
      : kind_(k), runs_(std::move(runs))
    {
        // FP32 density states are float pairs: the high planes, then the
        // low planes
        planes_ = (k.algo == ALGO_CVR) ? (k.N * k.N - 1) * (DF ? 2 : 1)
            : (k.algo == ALGO_CAYLEY)  ? k.N * k.N * (DF ? 2 : 1)
                                       : 0;
        // bound of the kernels' device-side waits (polls), and the test
        // switch that makes every persistent-kernel wait run out
        if (const char* w = std::getenv("MBG_WAIT_LIMIT")) wait_limit_ = (uint32_t) std::strtoul(w, nullptr, 10);
        if (const char* w = std::getenv("MBG_TEST_STALL_PERSIST")) stall_ = (w[0] == '1') ? (1u << 30) : 0u;
        MBG_CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        setup();
        choose_tuning(t);
    }

    ~engine_t()
    {
        for (int i = 0; i < 2; i++)
            if (graph_exec_[i]) cudaGraphExecDestroy(graph_exec_[i]);
        for (auto& e : events_) {
            cudaEventDestroy(e.a);
            cudaEventDestroy(e.b);
        }
        if (stream_) cudaStreamDestroy(stream_);
    }

    uint64_t steps_done() const override { return steps_done_; }
    uint64_t steps_total() const override { return nt_max_; }
    const run_setup& run(uint32_t r) const override { return runs_.at(r); }
    uint32_t num_runs() const override { return (uint32_t) runs_.size(); }
    uint64_t cells() const override { return cells_; }
    uint32_t tiles() const override { return (uint32_t) tiles_host_.size(); }
    tuning tuning_used() const override { return tune_; }
    int staging() const override { return staging_; }
    int persistent() const override { return persist_; }
    void set_timing(bool on) override { timing_ = on; }
    void restart_clock() override { steps_done_ = 0; }

    uint32_t status() override
    {
        uint32_t s = 0;
        MBG_CK(cudaStreamSynchronize(stream_));
        MBG_CK(cudaMemcpy(&s, status_.p, sizeof(s), cudaMemcpyDeviceToHost));
        return s;
    }

    void kernel_time(uint64_t* launches, double* ms, bool reset) override
    {
        MBG_CK(cudaStreamSynchronize(stream_));
        for (size_t i = ev_read_; i < ev_used_; i++) {
            float t = 0;
            MBG_CK(cudaEventElapsedTime(&t, events_[i].a, events_[i].b));
            acc_ms_ += t;
            acc_launches_ += events_[i].launches;
        }
        ev_read_ = ev_used_;
        *launches = acc_launches_;
        *ms = acc_ms_;
        if (reset) {
            acc_ms_ = 0;
            acc_launches_ = 0;
            ev_used_ = ev_read_ = 0;
        }
    }

    void advance(uint64_t steps) override
    {
        if (steps_done_ >= nt_max_) return;
        steps = std::min<uint64_t>(steps, nt_max_ - steps_done_);
        if (!steps) return;
        step_set_kernel<<<1, 1, 0, stream_>>>(step_.p, (unsigned long long) steps_done_);
        MBG_CK(cudaGetLastError());
        launches_ += 1;
        const uint64_t depth = tune_.depth;
        uint64_t full = steps / depth;
        const uint64_t rem = steps % depth;
        const uint32_t L = (uint32_t) tune_.graph;
        if (persist_) {
            // all full launches as persistent kernels; the levels of one
            // launch bounded so that its work items (levels x tiles, 32-bit
            // in the kernel) and the progress counters stay below 2^31
            const uint64_t per = std::max<uint64_t>(1, ((1ull << 31) - 1) / std::max<size_t>(1, tiles_host_.size()));
            while (full) {
                const uint32_t lv = (uint32_t) std::min<uint64_t>(std::min<uint64_t>(full, per), 1u << 20);
                launch_persistent(lv, (uint32_t) depth);
                full -= lv;
            }
        }
        if (L >= 2) {
            while (full >= L) {
                replay_graph();
                full -= L;
            }
        }
        for (uint64_t i = 0; i < full; i++) launch_group(1, (uint32_t) depth);
        if (rem) launch_group(1, (uint32_t) rem);
        steps_done_ += steps;
        MBG_CK(cudaGetLastError());
    }

    // ------------------------------------------------------ checkpoints
    struct state_header {
        char magic[8];
        uint32_t version, real_bytes, algo, levels;
        uint64_t n_total, planes, scratch, runs, nt_max, steps_done;
        uint64_t digest;  // of the run descriptions (describe_digest)
    };

    // FNV-1a (64 bit) over the descriptions that determine how a state
    // evolves: grid and step, boundary, materials (the precompute's FP64
    // inputs), regions, sources (with their tables) and records. Initial
    // conditions are left out: a checkpoint replaces the state they set.
    static uint64_t describe_digest(const std::vector<run_setup>& runs)
    {
        uint64_t h = 1469598103934665603ull;
        auto bytes = [&](const void* p, size_t n) {
            const unsigned char* c = static_cast<const unsigned char*>(p);
            for (size_t i = 0; i < n; i++) {
                h ^= c[i];
                h *= 1099511628211ull;
            }
        };
        auto num = [&](auto v) { bytes(&v, sizeof(v)); };
        num((uint64_t) runs.size());
        for (const run_setup& r : runs) {
            num(r.n_x), num(r.n_t), num(r.dx), num(r.dt), num(r.endtime);
            num(r.k_left), num(r.k_right);
            num((uint64_t) r.mats.size());
            for (const pre::mat_in& m : r.mats) {
                num(m.N), num(m.relax_kind), num(m.eps_r), num(m.mu_r), num(m.overlap), num(m.losses);
                num(m.carrier_density), num(m.dt), num(m.dx);
                bytes(m.h_re, sizeof(m.h_re)), bytes(m.h_im, sizeof(m.h_im));
                bytes(m.mu_re, sizeof(m.mu_re)), bytes(m.mu_im, sizeof(m.mu_im));
                bytes(m.S, sizeof(m.S)), bytes(m.deph, sizeof(m.deph));
            }
            for (const auto& g : r.regions) num(g.mat), num(g.x0), num(g.x1);
            for (const auto& s : r.sources) {
                num(s.type), num(s.shape), num(s.x_idx), num(s.on_grid), num(s.ampl), num(s.freq);
                num(s.phase), num(s.beta_or_tau), num(s.phase_sin);
                if (!s.table.empty()) bytes(s.table.data(), s.table.size() * sizeof(double));
            }
            for (const auto& c : r.records) {
                num(c.d.type), num(c.d.row_idx), num(c.d.col_idx), num(c.d.pos), num(c.d.cols);
                num(c.d.rows), num(c.d.ratio), num(c.is_complex), num(c.coherence);
            }
        }
        return h;
    }

    uint64_t state_bytes() const override
    {
        const uint64_t words = n_total_ * (3 + (DF ? 2 : 0)) + n_total_ * (uint64_t) planes_ + scratch_.n;
        return sizeof(state_header) + words * sizeof(T);
    }

    state_header header() const
    {
        state_header h{};
        std::memcpy(h.magic, "MBGSTATE", 8);
        h.version = 2;
        h.real_bytes = sizeof(T);
        h.algo = (uint32_t) kind_.algo;
        h.levels = (uint32_t) kind_.N;
        h.n_total = n_total_;
        h.planes = (uint64_t) planes_;
        h.scratch = scratch_.n;
        h.runs = runs_.size();
        h.nt_max = nt_max_;
        h.steps_done = steps_done_;
        h.digest = digest_;
        return h;
    }

    template<typename F>
    void state_arrays(F&& f)
    {
        f(E_[cur_].p, n_total_);
        f(H_[cur_].p, n_total_);
        f(P_[cur_].p, n_total_);
        if (DF) {
            f(El_[cur_].p, n_total_);
            f(Hl_[cur_].p, n_total_);
        }
        if (planes_) f(D_[cur_].p, n_total_ * (uint64_t) planes_);
        f(scratch_.p, (uint64_t) scratch_.n);
    }

    void save_state(void* host, uint64_t bytes) override
    {
        if (!host || bytes < state_bytes()) throw invalid_argument("state buffer too small");
        const state_header h = header();
        std::memcpy(host, &h, sizeof(h));
        char* o = static_cast<char*>(host) + sizeof(h);
        MBG_CK(cudaStreamSynchronize(stream_));
        state_arrays([&](T* p, uint64_t n) {
            MBG_CK(cudaMemcpy(o, p, n * sizeof(T), cudaMemcpyDeviceToHost));
            o += n * sizeof(T);
        });
    }

    void load_state(const void* host, uint64_t bytes) override
    {
        if (!host || bytes < sizeof(state_header)) throw invalid_argument("not a checkpoint");
        state_header h;
        std::memcpy(&h, host, sizeof(h));
        const state_header m = header();
        if (std::memcmp(h.magic, m.magic, 8) != 0 || h.version != m.version)
            throw invalid_argument("not a checkpoint");
        if (h.real_bytes != m.real_bytes || h.algo != m.algo || h.levels != m.levels || h.n_total != m.n_total ||
            h.planes != m.planes || h.scratch != m.scratch || h.runs != m.runs || h.nt_max != m.nt_max)
            throw invalid_argument("checkpoint does not match this ensemble");
        if (h.digest != m.digest)
            throw invalid_argument(
                "checkpoint belongs to an ensemble of other descriptions (grid, materials, sources or records)");
        if (bytes < state_bytes()) throw invalid_argument("checkpoint truncated");
        if (h.steps_done > nt_max_) throw invalid_argument("checkpoint step out of range");
        const char* i = static_cast<const char*>(host) + sizeof(h);
        MBG_CK(cudaStreamSynchronize(stream_));
        state_arrays([&](T* p, uint64_t n) {
            MBG_CK(cudaMemcpy(p, i, n * sizeof(T), cudaMemcpyHostToDevice));
            i += n * sizeof(T);
        });
        steps_done_ = h.steps_done;
    }

    void copy_result(uint32_t run, uint32_t k, double* re, double* im) override
    {
        const run_setup& rs = runs_.at(run);
        if (k >= rs.records.size()) throw invalid_argument("result index out of range");
        const auto& rc = rs.records[k];
        uint64_t size = (uint64_t) rc.d.cols * rc.d.rows;
        std::vector<T> tmp(size);
        MBG_CK(cudaStreamSynchronize(stream_));
        MBG_CK(cudaMemcpy(tmp.data(), scratch_.p + scratch_base_[run] + rc.d.offset,
                          size * sizeof(T), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < size; i++) re[i] = (double) tmp[i];
        if (im) {
            if (rc.is_complex) {
                MBG_CK(cudaMemcpy(tmp.data(), scratch_.p + scratch_base_[run] + rc.d.offset + size,
                                  size * sizeof(T), cudaMemcpyDeviceToHost));
                for (uint64_t i = 0; i < size; i++) im[i] = (double) tmp[i];
            } else {
                std::fill(im, im + size, 0.0);
            }
        }
    }

    void copy_probe_rows(uint32_t k, uint64_t row0, uint64_t nrows, double* out) override
    {
        const uint32_t nr = (uint32_t) runs_.size();
        std::vector<uint64_t> offs(nr);
        for (uint32_t r = 0; r < nr; r++) {
            const run_setup& rs = runs_[r];
            if (k >= rs.records.size() || rs.records[k].d.cols != 1)
                throw invalid_argument("record is not a single-point probe in every run");
            if (row0 + nrows > rs.records[k].d.rows) throw invalid_argument("rows out of range");
            offs[r] = scratch_base_[r] + rs.records[k].d.offset;
        }
        dbuf<uint64_t> doffs;
        doffs.alloc(nr);
        dbuf<T> tmp;
        tmp.alloc((size_t) nr * nrows);
        MBG_CK(cudaMemcpyAsync(doffs.p, offs.data(), nr * sizeof(uint64_t),
                               cudaMemcpyHostToDevice, stream_));
        gather_probe_kernel<T><<<1024, 256, 0, stream_>>>(scratch_.p, doffs.p, nr, row0, nrows, tmp.p);
        MBG_CK(cudaGetLastError());
        launches_ += 1;
        std::vector<T> h((size_t) nr * nrows);
        MBG_CK(cudaMemcpyAsync(h.data(), tmp.p, h.size() * sizeof(T), cudaMemcpyDeviceToHost, stream_));
        MBG_CK(cudaStreamSynchronize(stream_));
        for (size_t i = 0; i < h.size(); i++) out[i] = (double) h[i];
    }

private:
    struct ev_pair {
        cudaEvent_t a, b;
        uint64_t launches;
    };

    solver_kind kind_;
    std::vector<run_setup> runs_;
    int planes_ = 0;
    cudaStream_t stream_ = nullptr;
    uint64_t n_total_ = 0, cells_ = 0, nt_max_ = 0, steps_done_ = 0;
    std::vector<uint64_t> offsets_, scratch_base_;
    int mstride_ = 0, mstage_ = 0;
    int cur_ = 0;  // buffer holding the current state
    dbuf<T> E_[2], H_[2], P_[2], D_[2];
    dbuf<T> El_[2], Hl_[2];  // FP32: low parts of the double-float fields
    static constexpr bool DF = sizeof(T) == 4;
    dbuf<int32_t> mat_;
    dbuf<T> mc_, scratch_;
    dbuf<double> stab_;
    dbuf<double> mc64_;
    dbuf<run_desc> runs_dev_;
    dbuf<src_desc> srcs_;
    dbuf<rec_desc> recs_;
    dbuf<tile_desc> tiles_;
    // persistent kernel: tile neighbours, per-tile progress, work counter,
    // levels done since the tiles were built
    dbuf<int2> nb_;
    dbuf<uint32_t> prog_, work_;
    uint32_t pbase_ = 0;
    uint64_t digest_ = 0;  // describe_digest(runs_), for checkpoints
    uint32_t wait_limit_ = 0;  // MBG_WAIT_LIMIT (0: the kernels' defaults)
    uint32_t stall_ = 0;       // MBG_TEST_STALL_PERSIST
    persist_fn<T> pfn_ = nullptr;
    int persist_ = 0;
    dbuf<unsigned long long> step_, step_zero_;
    dbuf<uint32_t> status_;
    std::vector<tile_desc> tiles_host_;
    std::vector<run_desc> runs_host_;
    tuning tune_;
    launch_fn<T> fn_ = nullptr;
    cudaGraphExec_t graph_exec_[2] = { nullptr, nullptr };
    bool timing_ = false;
    std::vector<ev_pair> events_;
    size_t ev_used_ = 0, ev_read_ = 0;
    double acc_ms_ = 0;
    uint64_t acc_launches_ = 0;
    uint64_t launches_ = 0;  // every kernel launched by advance()/copies

    cudaEvent_t region_[2] = { nullptr, nullptr };

public:
    uint64_t launches() const override { return launches_; }

    double stream_time(bool begin) override
    {
        if (!region_[0]) {
            MBG_CK(cudaEventCreate(&region_[0]));
            MBG_CK(cudaEventCreate(&region_[1]));
        }
        if (begin) {
            MBG_CK(cudaEventRecord(region_[0], stream_));
            return 0.0;
        }
        MBG_CK(cudaEventRecord(region_[1], stream_));
        MBG_CK(cudaEventSynchronize(region_[1]));
        float ms = 0;
        MBG_CK(cudaEventElapsedTime(&ms, region_[0], region_[1]));
        return ms;
    }

private:

    void setup()
    {
        digest_ = describe_digest(runs_);
        const uint32_t nr = (uint32_t) runs_.size();
        if (nr == 0) throw invalid_argument("no runs");
        // packed ragged layout: runs back to back, 8-point aligned
        uint64_t off = GUARD_FRONT;
        for (const auto& r : runs_) {
            offsets_.push_back(off);
            off += ((uint64_t) r.n_x + 7) & ~7ull;
            cells_ += r.n_x;
            nt_max_ = std::max<uint64_t>(nt_max_, r.n_t);
        }
        n_total_ = ((off + GUARD_BACK) + 7) & ~7ull;
        for (int b = 0; b < 2; b++) {
            E_[b].alloc(n_total_);
            H_[b].alloc(n_total_);
            P_[b].alloc(n_total_);
            MBG_CK(cudaMemsetAsync(E_[b].p, 0, n_total_ * sizeof(T), stream_));
            MBG_CK(cudaMemsetAsync(H_[b].p, 0, n_total_ * sizeof(T), stream_));
            MBG_CK(cudaMemsetAsync(P_[b].p, 0, n_total_ * sizeof(T), stream_));
            if (planes_) {
                D_[b].alloc(n_total_ * planes_);
                MBG_CK(cudaMemsetAsync(D_[b].p, 0, n_total_ * planes_ * sizeof(T), stream_));
            }
            if (DF) {
                El_[b].alloc(n_total_);
                Hl_[b].alloc(n_total_);
                MBG_CK(cudaMemsetAsync(El_[b].p, 0, n_total_ * sizeof(T), stream_));
                MBG_CK(cudaMemsetAsync(Hl_[b].p, 0, n_total_ * sizeof(T), stream_));
            }
        }
        mat_.alloc(n_total_);
        MBG_CK(cudaMemsetAsync(mat_.p, 0xff, n_total_ * sizeof(int32_t), stream_));
        status_.alloc(1);
        MBG_CK(cudaMemsetAsync(status_.p, 0, sizeof(uint32_t), stream_));
        step_.alloc(1);
        step_zero_.alloc(1);
        MBG_CK(cudaMemsetAsync(step_.p, 0, sizeof(unsigned long long), stream_));
        MBG_CK(cudaMemsetAsync(step_zero_.p, 0, sizeof(unsigned long long), stream_));

        // materials: FP64 precompute on the GPU, one thread per material
        std::vector<pre::mat_in> mins;
        std::vector<uint32_t> mat_base;
        for (const auto& r : runs_) {
            mat_base.push_back((uint32_t) mins.size());
            mins.insert(mins.end(), r.mats.begin(), r.mats.end());
        }
        const int N = kind_.N;
        if (kind_.algo == ALGO_CVR) {
            mstride_ = pre::make_cvr_layout(N).stride;
            mstage_ = pre::make_cvr_layout(N).stage;
        } else if (kind_.algo == ALGO_CAYLEY) {
            // the FP64 kernels read only the leading part of the block
            mstride_ = pre::make_cay_layout(N).stride;
            mstage_ = DF ? mstride_ : pre::make_cay_layout(N).stage64;
        } else {
            mstride_ = pre::make_cvr_layout(0).stride;
            mstage_ = pre::make_cvr_layout(0).stage;
        }
        const size_t nm = std::max<size_t>(1, mins.size());
        size_t ws_stride = kind_.algo == ALGO_CVR ? pre::cvr_workspace(N)
            : kind_.algo == ALGO_CAYLEY            ? pre::cay_workspace(N)
                                                   : 1;
        {
            dbuf<pre::mat_in> din;
            din.alloc(nm);
            dbuf<double> ws;
            ws.alloc(nm * ws_stride);
            dbuf<int> codes;
            codes.alloc(nm);
            mc64_.alloc(nm * mstride_);
            MBG_CK(cudaMemcpyAsync(din.p, mins.data(), mins.size() * sizeof(pre::mat_in),
                                   cudaMemcpyHostToDevice, stream_));
            precompute_kernel<<<(unsigned) ((mins.size() + 63) / 64), 64, 0, stream_>>>(
                din.p, (int) mins.size(), kind_.algo, N, ws.p, ws_stride, mc64_.p, mstride_, codes.p);
            MBG_CK(cudaGetLastError());
            std::vector<int> hc(mins.size());
            MBG_CK(cudaMemcpyAsync(hc.data(), codes.p, hc.size() * sizeof(int),
                                   cudaMemcpyDeviceToHost, stream_));
            MBG_CK(cudaStreamSynchronize(stream_));
            for (int c : hc) {
                if (c == 1)
                    throw invalid_argument("Number of energy levels does not match selected solver!");
                if (c == 2) throw invalid_argument("Time-indepent matrix not invertible!");
                if (c == 3) throw invalid_argument("Unsupported superoperator!");
            }
        }
        mc_.alloc(nm * mstride_);
        cast_kernel<T><<<256, 256, 0, stream_>>>(mc64_.p, mc_.p, nm * mstride_);
        MBG_CK(cudaGetLastError());

        // initial state
        std::vector<init_desc> ids;
        std::vector<region_dev> regs;
        std::vector<double> evals, hvals;
        for (uint32_t r = 0; r < nr; r++) {
            const run_setup& rs = runs_[r];
            init_desc d;
            d.offset = offsets_[r];
            d.n_x = rs.n_x;
            d.dx = rs.dx;
            d.reg_begin = (uint32_t) regs.size();
            for (const auto& g : rs.regions) regs.push_back({ g.mat, g.x0, g.x1 });
            d.reg_end = (uint32_t) regs.size();
            d.mat_base = mat_base[r];
            d.e_kind = rs.e_kind;
            d.h_kind = rs.h_kind;
            d.e_val = rs.e_val;
            d.h_val = rs.h_val;
            d.e_off = evals.size();
            d.h_off = hvals.size();
            evals.insert(evals.end(), rs.e_vals.begin(), rs.e_vals.end());
            hvals.insert(hvals.end(), rs.h_vals.begin(), rs.h_vals.end());
            ids.push_back(d);
        }
        {
            dbuf<init_desc> dids;
            dids.alloc(ids.size());
            dbuf<region_dev> dregs;
            dregs.alloc(std::max<size_t>(1, regs.size()));
            dbuf<double> dev_e, dev_h;
            dev_e.alloc(std::max<size_t>(1, evals.size()));
            dev_h.alloc(std::max<size_t>(1, hvals.size()));
            MBG_CK(cudaMemcpyAsync(dids.p, ids.data(), ids.size() * sizeof(init_desc),
                                   cudaMemcpyHostToDevice, stream_));
            MBG_CK(cudaMemcpyAsync(dregs.p, regs.data(), regs.size() * sizeof(region_dev),
                                   cudaMemcpyHostToDevice, stream_));
            if (!evals.empty())
                MBG_CK(cudaMemcpyAsync(dev_e.p, evals.data(), evals.size() * sizeof(double),
                                       cudaMemcpyHostToDevice, stream_));
            if (!hvals.empty())
                MBG_CK(cudaMemcpyAsync(dev_h.p, hvals.data(), hvals.size() * sizeof(double),
                                       cudaMemcpyHostToDevice, stream_));
            dim3 grid(256, std::min<uint32_t>(nr, 65535));
            init_kernel<T><<<grid, 256, 0, stream_>>>(
                dids.p, nr, dregs.p, dev_e.p, dev_h.p, mc64_.p, mstride_, kind_.algo, N, planes_,
                mat_.p, E_[0].p, H_[0].p, P_[0].p, planes_ ? D_[0].p : nullptr, DF ? El_[0].p : nullptr,
                DF ? Hl_[0].p : nullptr, n_total_, status_.p);
            MBG_CK(cudaGetLastError());
            MBG_CK(cudaStreamSynchronize(stream_));
        }
        if (status() & STATUS_REGION) throw invalid_argument("region not found");

        // sources
        std::vector<src_desc> srcs;
        std::vector<srcgen_desc> gens;
        std::vector<double> tables;
        std::vector<uint64_t> table_dst;
        uint64_t tab_total = 0;
        runs_host_.resize(nr);
        for (uint32_t r = 0; r < nr; r++) {
            const run_setup& rs = runs_[r];
            run_desc& rd = runs_host_[r];
            rd.offset = offsets_[r];
            rd.n_x = rs.n_x;
            rd.n_t = rs.n_t;
            rd.dx_inv = 1.0 / rs.dx;
            rd.k_left = rs.k_left;
            rd.k_right = rs.k_right;
            rd.src_begin = (uint32_t) srcs.size();
            for (const auto& s : rs.sources) {
                if (!s.on_grid) continue;  // outside the grid: never applied
                src_desc d;
                d.type = s.type;
                d.x_idx = s.x_idx;
                d.table_offset = tab_total;
                if (s.shape == MBG_SHAPE_TABLE) {
                    table_dst.push_back(tab_total);
                    tables.insert(tables.end(), s.table.begin(), s.table.end());
                } else {
                    srcgen_desc g;
                    g.shape = s.shape;
                    g.n_t = rs.n_t;
                    g.dt = rs.dt;
                    g.ampl = s.ampl;
                    g.freq = s.freq;
                    g.phase = s.phase;
                    g.beta_or_tau = s.beta_or_tau;
                    g.phase_sin = s.phase_sin;
                    g.table_offset = tab_total;
                    gens.push_back(g);
                }
                tab_total += rs.n_t;
                srcs.push_back(d);
            }
            rd.src_end = (uint32_t) srcs.size();
        }
        stab_.alloc(std::max<uint64_t>(1, tab_total));
        srcs_.alloc(std::max<size_t>(1, srcs.size()));
        if (!srcs.empty())
            MBG_CK(cudaMemcpyAsync(srcs_.p, srcs.data(), srcs.size() * sizeof(src_desc),
                                   cudaMemcpyHostToDevice, stream_));
        if (!gens.empty()) {
            dbuf<srcgen_desc> dg;
            dg.alloc(gens.size());
            MBG_CK(cudaMemcpyAsync(dg.p, gens.data(), gens.size() * sizeof(srcgen_desc),
                                   cudaMemcpyHostToDevice, stream_));
            dim3 grid(64, std::min<size_t>(gens.size(), 65535));
            source_kernel<<<grid, 256, 0, stream_>>>(dg.p, (uint32_t) gens.size(), stab_.p);
            MBG_CK(cudaGetLastError());
            MBG_CK(cudaStreamSynchronize(stream_));
        }
        if (!tables.empty()) {
            // tabulated sources: FP64 values, cast on the device
            dbuf<double> dt;
            dt.alloc(tables.size());
            MBG_CK(cudaMemcpyAsync(dt.p, tables.data(), tables.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, stream_));
            // tables were concatenated in source order, n_t values each
            size_t pos = 0;
            size_t src_i = 0;
            for (uint32_t r = 0; r < nr; r++)
                for (const auto& s : runs_[r].sources) {
                    if (!s.on_grid || s.shape != MBG_SHAPE_TABLE) continue;
                    MBG_CK(cudaMemcpyAsync(stab_.p + table_dst[src_i], dt.p + pos,
                                           runs_[r].n_t * sizeof(double), cudaMemcpyDeviceToDevice,
                                           stream_));
                    pos += runs_[r].n_t;
                    src_i++;
                }
            MBG_CK(cudaStreamSynchronize(stream_));
        }

        // records: scratch per run, record offsets made absolute
        std::vector<rec_desc> recs;
        uint64_t sbase = 0;
        for (uint32_t r = 0; r < nr; r++) {
            run_desc& rd = runs_host_[r];
            scratch_base_.push_back(sbase);
            rd.rec_begin = (uint32_t) recs.size();
            for (const auto& rc : runs_[r].records) {
                rec_desc d = rc.d;
                d.offset += sbase;
                if (rc.coherence) {
                    d.type = REC_COH_RE;
                    recs.push_back(d);
                    d.type = REC_COH_IM;
                    d.offset += d.rows * d.cols;
                }
                recs.push_back(d);
            }
            rd.rec_end = (uint32_t) recs.size();
            sbase += runs_[r].scratch;
        }
        scratch_.alloc(std::max<uint64_t>(1, sbase));
        MBG_CK(cudaMemsetAsync(scratch_.p, 0, std::max<uint64_t>(1, sbase) * sizeof(T), stream_));
        recs_.alloc(std::max<size_t>(1, recs.size()));
        if (!recs.empty())
            MBG_CK(cudaMemcpyAsync(recs_.p, recs.data(), recs.size() * sizeof(rec_desc),
                                   cudaMemcpyHostToDevice, stream_));
        runs_dev_.alloc(nr);
        MBG_CK(cudaMemcpyAsync(runs_dev_.p, runs_host_.data(), nr * sizeof(run_desc),
                               cudaMemcpyHostToDevice, stream_));
        MBG_CK(cudaStreamSynchronize(stream_));
    }

    static int align_halo(int depth) { return (depth + 7) & ~7; }

    void build_tiles(const tuning& t)
    {
        const int halo = align_halo(t.depth);
        const int width = t.C * t.NT;
        const int out = width - 2 * halo;
        if (out <= 0) throw invalid_argument("tile too narrow for the temporal depth");
        tiles_host_.clear();
        for (uint32_t r = 0; r < runs_.size(); r++)
            for (int64_t s = 0; s < (int64_t) runs_[r].n_x; s += out)
                tiles_host_.push_back(
                    tile_desc{ r, (int32_t) s, (int32_t) std::min<int64_t>(out, runs_[r].n_x - s), -1 });
        tiles_.alloc(tiles_host_.size());
        MBG_CK(cudaMemcpyAsync(tiles_.p, tiles_host_.data(), tiles_host_.size() * sizeof(tile_desc),
                               cudaMemcpyHostToDevice, stream_));
        const unsigned nt = (unsigned) tiles_host_.size();
        tile_uniform_kernel<<<(nt + 7) / 8, 256, 0, stream_>>>(tiles_.p, nt, runs_dev_.p, mat_.p, halo);
        MBG_CK(cudaGetLastError());
        // persistent kernel: neighbours of each tile in its run, progress
        // counters from zero
        std::vector<int2> nb(nt);
        for (unsigned i = 0; i < nt; i++) {
            const bool l = i > 0 && tiles_host_[i - 1].run == tiles_host_[i].run;
            const bool r = i + 1 < nt && tiles_host_[i + 1].run == tiles_host_[i].run;
            nb[i] = make_int2(l ? (int) i - 1 : (int) i, r ? (int) i + 1 : (int) i);
        }
        nb_.alloc(std::max<size_t>(1, nt));
        prog_.alloc(std::max<size_t>(1, nt));
        MBG_CK(cudaMemcpyAsync(nb_.p, nb.data(), nt * sizeof(int2), cudaMemcpyHostToDevice, stream_));
        MBG_CK(cudaMemsetAsync(prog_.p, 0, std::max<size_t>(1, nt) * sizeof(uint32_t), stream_));
        if (!work_.p) work_.alloc(1);
        pbase_ = 0;
        MBG_CK(cudaStreamSynchronize(stream_));
        for (int i = 0; i < 2; i++)
            if (graph_exec_[i]) {
                cudaGraphExecDestroy(graph_exec_[i]);
                graph_exec_[i] = nullptr;
            }
    }

    launch_fn<T> find_kernel(int C, int NT) const
    {
        for (const auto& e : kernel_registry<T>())
            if (e.algo == kind_.algo && e.lev == kind_.N && e.C == C && e.NT == NT && e.staging == staging_ && e.fn)
                return e.fn;
        return nullptr;
    }

    // a shape may be registered twice (its persistent kernel compiled in a
    // translation unit of its own): the first entry with one
    persist_fn<T> find_persistent(int C, int NT) const
    {
        for (const auto& e : kernel_registry<T>())
            if (e.algo == kind_.algo && e.lev == kind_.N && e.C == C && e.NT == NT && e.staging == 0 && e.pfn)
                return e.pfn;
        return nullptr;
    }

    // MBG_PERSISTENT=1 / =0 force the persistent kernel on / off, as
    // mbg_tuning.persistent = 1 / 2 do; otherwise -1 (automatic)
    static int persistent_forced(const mbg_tuning* user)
    {
        if (user && user->persistent == 1) return 1;
        if (user && user->persistent == 2) return 0;
        const char* s = std::getenv("MBG_PERSISTENT");
        if (s && s[0] == '1') return 1;
        if (s && s[0] == '0') return 0;
        return -1;
    }

    // MBG_TILE_STAGING=bulk selects the kernels that stage the tile state in
    // shared memory with bulk (TMA) copies where such kernels exist (2-level
    // FP32); by default the state goes straight into registers, which
    // measured faster.
    static int staging_wanted()
    {
        const char* s = std::getenv("MBG_TILE_STAGING");
        return (s && std::string(s) == "bulk") ? 1 : 0;
    }

    int staging_ = 0;

    kparams<T> params(int in, uint32_t launch_idx, uint32_t nsub, bool record, const unsigned long long* step) const
    {
        kparams<T> p;
        const int out = 1 - in;
        p.Ein = E_[in].p;
        p.Hin = H_[in].p;
        p.Pin = P_[in].p;
        p.Din = planes_ ? D_[in].p : nullptr;
        p.Eout = E_[out].p;
        p.Hout = H_[out].p;
        p.Pout = P_[out].p;
        p.Dout = planes_ ? D_[out].p : nullptr;
        p.Elin = DF ? El_[in].p : nullptr;
        p.Hlin = DF ? Hl_[in].p : nullptr;
        p.Elout = DF ? El_[out].p : nullptr;
        p.Hlout = DF ? Hl_[out].p : nullptr;
        p.plane = n_total_;
        p.mat = mat_.p;
        p.mc = mc_.p;
        p.mstride = (uint32_t) mstride_;
        p.mstage = (uint32_t) mstage_;
        p.tiles = tiles_.p;
        p.runs = runs_dev_.p;
        p.srcs = srcs_.p;
        p.stab = stab_.p;
        p.recs = recs_.p;
        p.scratch = scratch_.p;
        p.step_base = step;
        p.launch_idx = launch_idx;
        p.depth = (uint32_t) tune_.depth;
        p.nsub = nsub;
        p.halo = (uint32_t) align_halo(tune_.depth);
        p.record = record ? 1 : 0;
        p.status = status_.p;
        p.wait_limit = wait_limit_;
        return p;
    }

    size_t smem() const { return (size_t) mstage_ * sizeof(T); }

    ev_pair& next_event()
    {
        if (ev_used_ == events_.size()) {
            ev_pair e;
            MBG_CK(cudaEventCreate(&e.a));
            MBG_CK(cudaEventCreate(&e.b));
            events_.push_back(e);
        }
        return events_[ev_used_++];
    }

    // `count` launches of nsub steps each, then advance the device clock
    void launch_group(uint32_t count, uint32_t nsub)
    {
        ev_pair* ev = nullptr;
        if (timing_) {
            ev = &next_event();
            ev->launches = count;
            MBG_CK(cudaEventRecord(ev->a, stream_));
        }
        for (uint32_t i = 0; i < count; i++) {
            kparams<T> p = params(cur_, i, nsub, true, step_.p);
            fn_(p, (unsigned) tiles_host_.size(), smem(), stream_);
            cur_ = 1 - cur_;
        }
        if (timing_) MBG_CK(cudaEventRecord(ev->b, stream_));
        step_bump_kernel<<<1, 1, 0, stream_>>>(step_.p, (unsigned long long) count * nsub);
        MBG_CK(cudaGetLastError());
        launches_ += count + 1;
    }

    // `levels` launches of nsub steps as one persistent kernel
    void launch_persistent(uint32_t levels, uint32_t nsub)
    {
        if ((uint64_t) pbase_ + levels >= (1ull << 31)) {
            // progress counters near wrapping: start them again from zero
            MBG_CK(cudaMemsetAsync(prog_.p, 0, prog_.n * sizeof(uint32_t), stream_));
            pbase_ = 0;
        }
        ev_pair* ev = nullptr;
        if (timing_) {
            ev = &next_event();
            ev->launches = levels;
            MBG_CK(cudaEventRecord(ev->a, stream_));
        }
        MBG_CK(cudaMemsetAsync(work_.p, 0, sizeof(uint32_t), stream_));
        persist_params q;
        q.levels = levels;
        q.n_tiles = (uint32_t) tiles_host_.size();
        q.base = pbase_;
        q.work = work_.p;
        q.prog = prog_.p;
        q.nb = nb_.p;
        q.wait_limit = wait_limit_;
        q.stall = stall_;
        // level k reads buffer cur_ ^ (k & 1): the kernel flips odd levels
        kparams<T> p = params(cur_, 0, nsub, true, step_.p);
        pfn_(p, q, smem(), stream_);
        MBG_CK(cudaGetLastError());
        if (timing_) MBG_CK(cudaEventRecord(ev->b, stream_));
        if (levels & 1u) cur_ = 1 - cur_;
        pbase_ += levels;
        step_bump_kernel<<<1, 1, 0, stream_>>>(step_.p, (unsigned long long) levels * nsub);
        MBG_CK(cudaGetLastError());
        launches_ += 3;
    }

    void replay_graph()
    {
        const uint32_t L = (uint32_t) tune_.graph;
        if (!graph_exec_[cur_]) {
            cudaGraph_t g;
            const int start = cur_;
            MBG_CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
            int c = cur_;
            for (uint32_t i = 0; i < L; i++) {
                kparams<T> p = params(c, i, (uint32_t) tune_.depth, true, step_.p);
                fn_(p, (unsigned) tiles_host_.size(), smem(), stream_);
                c = 1 - c;
            }
            step_bump_kernel<<<1, 1, 0, stream_>>>(step_.p, (unsigned long long) L * tune_.depth);
            MBG_CK(cudaStreamEndCapture(stream_, &g));
            MBG_CK(cudaGraphInstantiate(&graph_exec_[start], g, 0));
            cudaGraphDestroy(g);
        }
        ev_pair* ev = nullptr;
        if (timing_) {
            ev = &next_event();
            ev->launches = L;
            MBG_CK(cudaEventRecord(ev->a, stream_));
        }
        MBG_CK(cudaGraphLaunch(graph_exec_[cur_], stream_));
        launches_ += L + 1;
        if (timing_) MBG_CK(cudaEventRecord(ev->b, stream_));
        if (L % 2) cur_ = 1 - cur_;
    }

    // ------------------------------------------------------ autotuner

    std::string tune_key() const
    {
        std::ostringstream s;
        int dev = 0;
        cudaDeviceProp prop;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
            for (const char* c = prop.name; *c; c++) s << (std::isalnum((unsigned char) *c) ? *c : '_');
            s << "_" << prop.multiProcessorCount << ":";
        }
        s << kind_.algo << ":" << kind_.N << ":s" << staging_ << ":" << (kind_.fp64 ? 64 : 32) << ":"
          << (cells_ >> 16) << ":" << runs_.size() << ":" << std::min<uint64_t>(nt_max_, 256);
        return s.str();
    }

    tuning default_tuning() const
    {
        tuning t;
        const bool d = kind_.fp64;
        if (kind_.algo == ALGO_NOOP) {
            t.C = d ? 4 : 8;
            t.NT = 256;
            t.depth = 16;
        } else if (kind_.algo == ALGO_CVR) {
            if (kind_.N == 2) {
                t.C = d ? 2 : 4;
                t.NT = 256;
                t.depth = d ? 8 : 16;
            } else if (kind_.N == 3) {
                t.C = d ? 1 : 2;
                t.NT = 128;
                t.depth = 8;
            } else {
                t.C = 1;
                t.NT = 128;
                t.depth = 4;
            }
        } else {
            if (kind_.N == 2) {
                t.C = 2;
                t.NT = 256;
                t.depth = 8;
            } else if (kind_.N == 3) {
                t.C = 1;
                t.NT = 128;
                t.depth = 8;
            } else {
                t.C = 1;
                t.NT = 128;
                t.depth = 4;
            }
        }
        t.graph = 8;
        return t;
    }

    double time_candidate(const tuning& t, int reps = 3)
    {
        tune_ = t;
        fn_ = find_kernel(t.C, t.NT);
        if (!fn_) return -1.0;
        build_tiles(t);
        // reads the current state, writes the other buffer: no state change
        auto once = [&]() {
            kparams<T> p = params(cur_, 0, (uint32_t) t.depth, false, step_zero_.p);
            fn_(p, (unsigned) tiles_host_.size(), smem(), stream_);
        };
        once();
        MBG_CK(cudaGetLastError());
        cudaEvent_t a, b;
        MBG_CK(cudaEventCreate(&a));
        MBG_CK(cudaEventCreate(&b));
        MBG_CK(cudaEventRecord(a, stream_));
        for (int i = 0; i < reps; i++) once();
        MBG_CK(cudaEventRecord(b, stream_));
        MBG_CK(cudaEventSynchronize(b));
        float ms = 0;
        MBG_CK(cudaEventElapsedTime(&ms, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        MBG_CK(cudaGetLastError());
        const double steps = std::min<double>(t.depth, (double) nt_max_);
        return (double) cells_ * steps * reps / (ms * 1e-3);
    }

    // Close contenders (within `margin` of the best first timing) are timed
    // again, round-robin over several trials so that clock or thermal drift
    // affects them alike, and the best of each one's trials decides: a
    // single short timing cannot separate shapes a few per cent apart.
    tuning runoff(const std::vector<std::pair<tuning, double> >& first, double margin)
    {
        double top = 0;
        for (const auto& c : first) top = std::max(top, c.second);
        std::vector<tuning> cands;
        for (const auto& c : first)
            if (c.second >= top * (1.0 - margin)) cands.push_back(c.first);
        std::vector<double> best(cands.size(), 0.0);
        if (cands.size() > 1)
            for (int trial = 0; trial < 3; trial++)
                for (size_t i = 0; i < cands.size(); i++) best[i] = std::max(best[i], time_candidate(cands[i], 4));
        size_t bi = 0;
        for (size_t i = 1; i < cands.size(); i++)
            if (best[i] > best[bi]) bi = i;
        return cands[bi];
    }

    // The depth timings are of the launch per level, whose launches lose
    // the unfilled part of their last wave of tiles; the persistent kernel
    // does not. Where the persistent kernel will run, rank the depths by
    // their rate divided by that wave efficiency, tiles / (ceil(tiles /
    // slots) * slots): one 65,536-point 6-level run measured 8.4e9
    // cell-updates/s persistent at depth 8 (launch per level 5.8e9, 1.29
    // waves) and 8.0e9 at depth 16 (6.3e9, 1.50 waves), which this ranks
    // 9.0 vs 8.4.
    tuning persistent_depth(const tuning& best, const std::vector<std::pair<tuning, double> >& depths,
                            const std::vector<size_t>& ntiles, int forced)
    {
        if (forced == 0 || staging_ != 0 || depths.size() < 2) return best;
        persist_fn<T> pf = find_persistent(best.C, best.NT);
        if (!pf) return best;
        fn_ = find_kernel(best.C, best.NT);
        persist_params q{};
        const double slots = (double) pf(params(cur_, 0, 1, false, step_zero_.p), q, smem(), stream_);
        if (slots < 1) return best;
        tuning pick = best;
        double top = -1.0;
        for (size_t i = 0; i < depths.size(); i++) {
            const double n = (double) ntiles[i];
            if (depths[i].second <= 0 || n <= 0) continue;
            if (forced < 0 && n >= 4 * slots) continue;  // would not run persistent
            const double eff = n / (std::ceil(n / slots) * slots);
            const double est = depths[i].second / eff;
            if (est > top) {
                top = est;
                pick = depths[i].first;
            }
        }
        return pick;
    }

    void choose_tuning(const mbg_tuning* user)
    {
        staging_ = 0;
        if (staging_wanted() || (user && user->staging == 1))
            for (const auto& e : kernel_registry<T>())
                if (e.algo == kind_.algo && e.lev == kind_.N && e.staging == 1) staging_ = 1;
        tuning t = default_tuning();
        bool explicit_all = user && user->cells_per_thread && user->threads && user->depth;
        if (user) {
            if (user->cells_per_thread) t.C = (int) user->cells_per_thread;
            if (user->threads) t.NT = (int) user->threads;
            if (user->depth) t.depth = (int) user->depth;
            if (user->launches_per_graph) t.graph = (int) user->launches_per_graph;
        }
        if (t.depth < 1 || t.depth > MAX_DEPTH) throw invalid_argument("temporal depth must be 1..256");
        const char* env = std::getenv("MBG_AUTOTUNE");
        const bool autotune = !explicit_all && !(env && env[0] == '0');
        if (autotune) {
            std::string key = tune_key();
            bool cached = false;
            {
                std::lock_guard<std::mutex> lk(g_tune_mutex);
                tune_file_read();
                auto it = g_tune_cache.find(key);
                if (it != g_tune_cache.end()) {
                    t = it->second;
                    cached = true;
                }
            }
            if (!cached) {
                // stage 1: launch shape at the default depth; stage 2: depth
                // (each stage ends with a run-off of its close contenders)
                std::vector<std::pair<tuning, double> > shapes;
                for (const auto& e : kernel_registry<T>()) {
                    if (e.algo != kind_.algo || e.lev != kind_.N || e.staging != staging_ || !e.fn) continue;
                    tuning c = t;
                    c.C = e.C;
                    c.NT = e.NT;
                    if (align_halo(c.depth) * 4 > c.C * c.NT) continue;
                    shapes.push_back({ c, time_candidate(c) });
                }
                tuning best = shapes.empty() ? t : runoff(shapes, 0.10);
                std::vector<std::pair<tuning, double> > depths;
                std::vector<size_t> ntiles;
                for (int d : { 1, 2, 4, 8, 16, 32, 64 }) {
                    tuning c = best;
                    c.depth = d;
                    if (align_halo(d) * 4 > c.C * c.NT) continue;
                    if (d > 1 && (uint64_t) d > nt_max_) continue;
                    depths.push_back({ c, time_candidate(c) });
                    ntiles.push_back(tiles_host_.size());
                }
                if (!depths.empty()) best = runoff(depths, 0.05);
                best = persistent_depth(best, depths, ntiles, persistent_forced(user));
                t = best;
                std::lock_guard<std::mutex> lk(g_tune_mutex);
                g_tune_cache[key] = t;
                tune_file_append(key, t);
            }
        }
        if (t.graph % 2) t.graph += 1;
        tune_ = t;
        fn_ = find_kernel(t.C, t.NT);
        if (!fn_) {
            std::ostringstream s;
            s << "no kernel instantiated for cells_per_thread=" << t.C << " threads=" << t.NT;
            throw invalid_argument(s.str());
        }
        pfn_ = staging_ == 0 ? find_persistent(t.C, t.NT) : nullptr;
        build_tiles(t);
        persist_ = 0;
        if (pfn_) {
            const int forced = persistent_forced(user);
            if (forced >= 0) {
                persist_ = forced;
            } else {
                // automatic: with few waves of tiles per launch the launch
                // tails and the gaps between launches cost most (one
                // 65,536-point 6-level run: 1.3 waves, 5.8e9 -> 8.4e9
                // cell-updates/s persistent); with many the per-tile hand-off
                // costs more than it saves (4,096 2-level runs: 12 % slower)
                persist_params q{};
                const unsigned slots = pfn_(params(cur_, 0, 1, false, step_zero_.p), q, smem(), stream_);
                persist_ = tiles_host_.size() < 4ull * slots ? 1 : 0;
            }
        }
    }
};

std::unique_ptr<engine> make_engine(const solver_kind& k, std::vector<run_setup>&& runs, const mbg_tuning* t)
{
    if (k.fp64) return std::unique_ptr<engine>(new engine_t<double>(k, std::move(runs), t));
    return std::unique_ptr<engine>(new engine_t<float>(k, std::move(runs), t));
}

}  // namespace mbg
