// The C-ABI of include/mbsolve_gb300.h. No exception crosses it: every
// entry point returns a status and keeps the message for mbg_last_error().
#include <cstring>
#include <sstream>
#include <string>

#include "engine.hpp"

namespace {

thread_local std::string g_last_error;

template<typename F>
int guarded(F&& f)
{
    try {
        f();
        return MBG_OK;
    } catch (const mbg::cuda_error& e) {
        g_last_error = e.what();
        return MBG_ERR_CUDA;
    } catch (const std::invalid_argument& e) {
        g_last_error = e.what();
        return MBG_ERR_INVALID_ARGUMENT;
    } catch (const std::bad_alloc& e) {
        g_last_error = std::string("host allocation failed: ") + e.what();
        return MBG_ERR_RUNTIME;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return MBG_ERR_RUNTIME;
    }
}

// Device status after a complete run: a wait that ran out or a recorded
// NaN/Inf ends the call with MBG_ERR_RUNTIME (the results stay readable).
void check_status(uint32_t st)
{
    if (st & mbg::STATUS_TC_WAIT)
        throw std::runtime_error("CUDA: a tensor-core or bulk-copy completion wait ran out");
    if (st & mbg::STATUS_PERSIST_WAIT)
        throw std::runtime_error("CUDA: a persistent-kernel wait for neighbour tiles ran out");
    if (st & mbg::STATUS_NONFINITE)
        throw std::runtime_error("non-finite value (NaN or Inf) recorded: the simulation diverged");
}

void fill_grid(const mbg::run_setup& r, mbg_grid* g)
{
    g->num_gridpoints = r.n_x;
    g->num_timesteps = r.n_t;
    g->gridpoint_size = r.dx;
    g->timestep_size = r.dt;
    g->endtime = r.endtime;
}

}  // namespace

namespace mbg {
// lets entry points defined in other files report through mbg_last_error()
void set_last_error(const char* msg) { g_last_error = msg; }
}  // namespace mbg

struct mbg_solver {
    std::unique_ptr<mbg::engine> eng;
};

struct mbg_ensemble {
    std::unique_ptr<mbg::engine> eng;
};

extern "C" {

const char* mbg_version(void) { return "mbsolve_gb300 0.1.0 (sm_103a)"; }

const char* mbg_last_error(void) { return g_last_error.c_str(); }

size_t mbg_solver_names(char* buf, size_t len)
{
    std::string s;
    for (const auto& n : mbg::solver_names()) {
        if (!s.empty()) s += "\n";
        s += n;
    }
    if (buf && len) {
        size_t c = std::min(len - 1, s.size());
        std::memcpy(buf, s.data(), c);
        buf[c] = 0;
    }
    return s.size() + 1;
}

int mbg_scenario_grid(const mbg_device* dev, const mbg_scenario* scen, mbg_grid* out)
{
    return guarded([&] {
        if (!out) throw mbg::invalid_argument("null argument");
        mbg::solver_kind k;
        k.algo = mbg::ALGO_NOOP;
        k.N = 0;
        k.fp64 = true;
        fill_grid(mbg::setup_run(k, dev, scen), out);
    });
}

int mbg_solver_create(
    const char* name,
    const mbg_device* dev,
    const mbg_scenario* scen,
    const mbg_tuning* tuning,
    mbg_solver** out)
{
    return guarded([&] {
        if (!name || !out) throw mbg::invalid_argument("null argument");
        *out = nullptr;
        mbg::solver_kind k;
        if (!mbg::parse_solver_name(name, k))
            throw mbg::invalid_argument(std::string("Unknown solver ") + name);
        std::vector<mbg::run_setup> runs;
        runs.push_back(mbg::setup_run(k, dev, scen));
        auto* s = new mbg_solver();
        try {
            s->eng = mbg::make_engine(k, std::move(runs), tuning);
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
    });
}

int mbg_solver_grid(const mbg_solver* s, mbg_grid* out)
{
    return guarded([&] {
        if (!s || !out) throw mbg::invalid_argument("null argument");
        fill_grid(s->eng->run(0), out);
    });
}

int mbg_solver_run(mbg_solver* s)
{
    return guarded([&] {
        if (!s) throw mbg::invalid_argument("null argument");
        // like solver_cpu_fdtd::run: n_t steps from the current state,
        // time index (sources, record rows) starting at 0
        s->eng->restart_clock();
        s->eng->advance(s->eng->steps_total());
        check_status(s->eng->status());
    });
}

int mbg_solver_num_results(const mbg_solver* s, uint32_t* n)
{
    return guarded([&] {
        if (!s || !n) throw mbg::invalid_argument("null argument");
        *n = (uint32_t) s->eng->run(0).records.size();
    });
}

int mbg_solver_result_shape(
    const mbg_solver* s,
    uint32_t k,
    uint32_t* rows,
    uint32_t* cols,
    int32_t* is_complex)
{
    return guarded([&] {
        if (!s) throw mbg::invalid_argument("null argument");
        const auto& r = s->eng->run(0);
        if (k >= r.records.size()) throw mbg::invalid_argument("result index out of range");
        if (rows) *rows = (uint32_t) r.records[k].d.rows;
        if (cols) *cols = r.records[k].d.cols;
        if (is_complex) *is_complex = r.records[k].is_complex;
    });
}

int mbg_solver_copy_result(const mbg_solver* s, uint32_t k, double* real, double* imag)
{
    return guarded([&] {
        if (!s || !real) throw mbg::invalid_argument("null argument");
        s->eng->copy_result(0, k, real, imag);
    });
}

void mbg_solver_destroy(mbg_solver* s) { delete s; }

int mbg_ensemble_create(
    const char* name,
    uint32_t num_runs,
    const mbg_device* const* devs,
    const mbg_scenario* const* scens,
    const mbg_tuning* tuning,
    mbg_ensemble** out)
{
    return guarded([&] {
        if (!name || !out || !devs || !scens) throw mbg::invalid_argument("null argument");
        *out = nullptr;
        mbg::solver_kind k;
        if (!mbg::parse_solver_name(name, k))
            throw mbg::invalid_argument(std::string("Unknown solver ") + name);
        if (num_runs == 0) throw mbg::invalid_argument("an ensemble needs at least one run");
        std::vector<mbg::run_setup> runs;
        runs.reserve(num_runs);
        for (uint32_t i = 0; i < num_runs; i++) runs.push_back(mbg::setup_run(k, devs[i], scens[i]));
        auto* e = new mbg_ensemble();
        try {
            e->eng = mbg::make_engine(k, std::move(runs), tuning);
        } catch (...) {
            delete e;
            throw;
        }
        *out = e;
    });
}

int mbg_ensemble_advance(mbg_ensemble* e, uint32_t n_steps)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        e->eng->advance(n_steps);
    });
}

int mbg_ensemble_run(mbg_ensemble* e)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        e->eng->advance(e->eng->steps_total());
        check_status(e->eng->status());
    });
}

int mbg_ensemble_progress(const mbg_ensemble* e, uint64_t* done, uint64_t* total)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        if (done) *done = e->eng->steps_done();
        if (total) *total = e->eng->steps_total();
    });
}

int mbg_ensemble_grid(const mbg_ensemble* e, uint32_t run, mbg_grid* out)
{
    return guarded([&] {
        if (!e || !out) throw mbg::invalid_argument("null argument");
        if (run >= e->eng->num_runs()) throw mbg::invalid_argument("run index out of range");
        fill_grid(e->eng->run(run), out);
    });
}

int mbg_ensemble_result_shape(
    const mbg_ensemble* e,
    uint32_t run,
    uint32_t k,
    uint32_t* rows,
    uint32_t* cols,
    int32_t* is_complex)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        if (run >= e->eng->num_runs()) throw mbg::invalid_argument("run index out of range");
        const auto& r = e->eng->run(run);
        if (k >= r.records.size()) throw mbg::invalid_argument("result index out of range");
        if (rows) *rows = (uint32_t) r.records[k].d.rows;
        if (cols) *cols = r.records[k].d.cols;
        if (is_complex) *is_complex = r.records[k].is_complex;
    });
}

int mbg_ensemble_copy_result(
    const mbg_ensemble* e,
    uint32_t run,
    uint32_t k,
    double* real,
    double* imag)
{
    return guarded([&] {
        if (!e || !real) throw mbg::invalid_argument("null argument");
        if (run >= e->eng->num_runs()) throw mbg::invalid_argument("run index out of range");
        e->eng->copy_result(run, k, real, imag);
    });
}

int mbg_ensemble_copy_probe_rows(
    const mbg_ensemble* e,
    uint32_t k,
    uint64_t row0,
    uint64_t nrows,
    double* out)
{
    return guarded([&] {
        if (!e || !out) throw mbg::invalid_argument("null argument");
        e->eng->copy_probe_rows(k, row0, nrows, out);
    });
}

int mbg_ensemble_info(const mbg_ensemble* e, uint64_t* cells, uint32_t* tiles, mbg_tuning* t)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        if (cells) *cells = e->eng->cells();
        if (tiles) *tiles = e->eng->tiles();
        if (t) {
            mbg::tuning u = e->eng->tuning_used();
            t->cells_per_thread = (uint32_t) u.C;
            t->threads = (uint32_t) u.NT;
            t->depth = (uint32_t) u.depth;
            t->launches_per_graph = (uint32_t) u.graph;
            t->staging = (uint32_t) e->eng->staging();
            t->persistent = (uint32_t) e->eng->persistent();
        }
    });
}

int mbg_ensemble_set_timing(mbg_ensemble* e, int enable)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        e->eng->set_timing(enable != 0);
    });
}

int mbg_ensemble_kernel_time(mbg_ensemble* e, uint64_t* launches, double* ms, int reset)
{
    return guarded([&] {
        if (!e || !launches || !ms) throw mbg::invalid_argument("null argument");
        e->eng->kernel_time(launches, ms, reset != 0);
    });
}

int mbg_ensemble_stream_time(mbg_ensemble* e, int begin, double* ms)
{
    return guarded([&] {
        if (!e || (!begin && !ms)) throw mbg::invalid_argument("null argument");
        double t = e->eng->stream_time(begin != 0);
        if (!begin) *ms = t;
    });
}

int mbg_ensemble_launches(const mbg_ensemble* e, uint64_t* launches)
{
    return guarded([&] {
        if (!e || !launches) throw mbg::invalid_argument("null argument");
        *launches = e->eng->launches();
    });
}

int mbg_ensemble_state_size(const mbg_ensemble* e, uint64_t* bytes)
{
    return guarded([&] {
        if (!e || !bytes) throw mbg::invalid_argument("null argument");
        *bytes = e->eng->state_bytes();
    });
}

int mbg_ensemble_save_state(mbg_ensemble* e, void* host, uint64_t bytes)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        e->eng->save_state(host, bytes);
    });
}

int mbg_ensemble_load_state(mbg_ensemble* e, const void* host, uint64_t bytes)
{
    return guarded([&] {
        if (!e) throw mbg::invalid_argument("null argument");
        e->eng->load_state(host, bytes);
    });
}

int mbg_ensemble_status(mbg_ensemble* e, uint32_t* flags)
{
    return guarded([&] {
        if (!e || !flags) throw mbg::invalid_argument("null argument");
        *flags = e->eng->status();
    });
}

void mbg_ensemble_destroy(mbg_ensemble* e) { delete e; }

int mbg_material_constants(
    const char* algo,
    const mbg_material* mat,
    double timestep,
    int on_device,
    double* out,
    size_t cap,
    size_t* len)
{
    return guarded([&] {
        if (!algo || !mat || !len) throw mbg::invalid_argument("null argument");
        std::string a(algo);
        int kind = a == "cvr-rodr" ? mbg::ALGO_CVR : a == "reg-cayley" ? mbg::ALGO_CAYLEY : -1;
        if (kind < 0) throw mbg::invalid_argument("algo must be cvr-rodr or reg-cayley");
        // one-point device of this material, dx = 1 m
        mbg_region reg{ 0, 0.0, 1.0 };
        mbg_device dev{ 1, mat, 1, &reg };
        mbg_scenario sc;
        std::memset(&sc, 0, sizeof(sc));
        sc.num_gridpoints = 1;
        sc.endtime = timestep;
        sc.num_timesteps = 2;
        mbg::solver_kind k;
        k.algo = (mbg::algo_t) kind;
        k.N = mat->qm ? (int) mat->qm->num_levels : 2;
        k.fp64 = true;
        mbg::run_setup r = mbg::setup_run(k, &dev, &sc);
        mbg::pre::mat_in in = r.mats[0];
        in.dt = timestep;
        in.dx = 1.0;
        const int N = k.N;
        int stride = kind == mbg::ALGO_CVR ? mbg::pre::make_cvr_layout(N).stride
                                           : mbg::pre::make_cay_layout(N).stride;
        size_t ws_n = kind == mbg::ALGO_CVR ? mbg::pre::cvr_workspace(N) : mbg::pre::cay_workspace(N);
        *len = (size_t) stride;
        if (!out || cap < (size_t) stride) return;
        std::vector<double> res(stride);
        int code = 0;
        if (on_device) {
            mbg::pre::mat_in* din;
            double *ws, *dout;
            int* dcode;
            MBG_CK(cudaMalloc((void**) &din, sizeof(in)));
            MBG_CK(cudaMalloc((void**) &ws, ws_n * sizeof(double)));
            MBG_CK(cudaMalloc((void**) &dout, stride * sizeof(double)));
            MBG_CK(cudaMalloc((void**) &dcode, sizeof(int)));
            MBG_CK(cudaMemcpy(din, &in, sizeof(in), cudaMemcpyHostToDevice));
            mbg::launch_precompute(din, 1, kind, N, ws, ws_n, dout, stride, dcode, 0);
            MBG_CK(cudaGetLastError());
            MBG_CK(cudaMemcpy(res.data(), dout, stride * sizeof(double), cudaMemcpyDeviceToHost));
            MBG_CK(cudaMemcpy(&code, dcode, sizeof(int), cudaMemcpyDeviceToHost));
            cudaFree(din);
            cudaFree(ws);
            cudaFree(dout);
            cudaFree(dcode);
        } else {
            std::vector<double> ws(ws_n);
            code = kind == mbg::ALGO_CVR ? mbg::pre::cvr_precompute(in, N, ws.data(), res.data())
                                         : mbg::pre::cay_precompute(in, N, ws.data(), res.data());
        }
        if (code == 1) throw mbg::invalid_argument("Number of energy levels does not match selected solver!");
        if (code == 2) throw mbg::invalid_argument("Time-indepent matrix not invertible!");
        if (code == 3) throw mbg::invalid_argument("Unsupported superoperator!");
        std::memcpy(out, res.data(), stride * sizeof(double));
    });
}

size_t mbg_material_layout(const char* algo, uint32_t N, char* buf, size_t len)
{
    std::ostringstream s;
    std::string a(algo ? algo : "");
    if (a == "cvr-rodr") {
        mbg::pre::cvr_layout L = mbg::pre::make_cvr_layout((int) N);
        s << "V=" << L.V << "\nKP=" << L.KP << "\na=" << L.a << "\nb=" << L.b << "\ncH=" << L.cH
          << "\ngamma=" << L.gam << "\nhas_qm=" << L.has_qm << "\np0=" << L.p0 << "\nnplanes=" << L.nplanes
          << "\nBd=" << L.Bd << "\nBdl=" << L.Bdl << "\nk=" << L.k << "\ng=" << L.g << "\nthdt=" << L.thdt
          << "\nu0=" << L.z0 << "\nbdx=" << mbg::pre::FD_BDX << "\nbdx_lo=" << mbg::pre::FD_BDX_LO
          << "\ncH_lo=" << mbg::pre::FD_C_LO << "\nbG=" << mbg::pre::FD_G
          << "\ninv=" << L.inv << "\ninv_c=" << L.inv_c << "\npop=" << L.pop << "\npop_c=" << L.pop_c
          << "\nQ=" << L.Q << "\nBh=" << L.Bh << "\nkh=" << L.kh << "\ncoh=" << L.coh << "\ncoh_c=" << L.coh_c << "\nstage=" << L.stage << "\nstride=" << L.stride;
    } else if (a == "reg-cayley") {
        mbg::pre::cay_layout L = mbg::pre::make_cay_layout((int) N);
        s << "a=" << L.a << "\nb=" << L.b << "\ncH=" << L.cH << "\ngamma=" << L.gam << "\nhas_qm=" << L.has_qm
          << "\nkH0=" << L.kH0 << "\nkMu=" << L.kMu << "\nW0=" << L.W0 << "\nMn=" << L.Mn << "\ndD1=" << L.dD1
          << "\nd1=" << L.d1 << "\ndD2=" << L.dD2 << "\nd2=" << L.d2 << "\nrho0=" << L.rho0
          << "\ngP=" << L.gP << "\nstage64=" << L.stage64 << "\nU0=" << L.U0 << "\nWk=" << L.Wk
          << "\nNP=" << L.NP << "\nB0=" << L.B0 << "\nB0l=" << L.B0l << "\nblockB0=" << L.blockB0
          << "\nstride=" << L.stride;
    }
    std::string t = s.str();
    if (buf && len) {
        size_t c = std::min(len - 1, t.size());
        std::memcpy(buf, t.data(), c);
        buf[c] = 0;
    }
    return t.size() + 1;
}

}  // extern "C"
