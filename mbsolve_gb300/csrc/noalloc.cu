// Allocation-free variant of the per-material FP64 precompute.
//
// Some callers cannot call cudaMalloc: programs whose device memory is all
// owned by another allocator (a host framework's memory pool, or a process
// that reserves the GPU's memory up front), and code paths that must not
// pay the device-wide synchronisation cudaMalloc/cudaFree imply. For them,
// mbg_material_constants_noalloc() computes a material's constant block
// into a device buffer the caller provides, and keeps the precompute's FP64
// workspace in the fixed array below instead of allocating one.
//
// The array is a file-scope __device__ variable: every GPU that loads this
// library holds it (NOALLOC_WS_DOUBLES doubles, about 160 KB) until the
// process exits. All calls share it and it keeps the previous call's
// contents: the precompute writes every workspace entry before reading it,
// and the status slot is cleared by each call's kernel before anything
// else. Calls that overlap on the GPU (different streams, different host
// threads) race on the array and must not be issued.
#include <cstring>
#include <string>

#include "engine.hpp"
#include "precompute.cuh"

namespace {

// Largest workspace the precompute needs: the coherence-vector form at the
// largest level count (6 levels, 35 x 35 matrices), plus one status slot.
constexpr size_t NOALLOC_WS_DOUBLES = 20480;
constexpr size_t NOALLOC_STATUS_SLOT = NOALLOC_WS_DOUBLES - 1;

static __device__ __align__(256) double g_noalloc_ws[NOALLOC_WS_DOUBLES];

__global__ void precompute_noalloc_kernel(
    const mbg::pre::mat_in m,
    int algo,
    int N,
    double* ws,
    double* out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int* code = reinterpret_cast<int*>(ws + NOALLOC_STATUS_SLOT);
    *code = -1;  // cleared first: the slot holds the previous call's value
    int rc;
    if (algo == mbg::ALGO_CVR)
        rc = mbg::pre::cvr_precompute(m, N, ws, out);
    else
        rc = mbg::pre::cay_precompute(m, N, ws, out);
    *code = rc;
}

// Device address of g_noalloc_ws on the current device. The host-side
// symbol is only a stand-in, not an address a kernel can use. It is looked
// up on every call, with the call's device current: a cached address would
// go stale when the device's context is destroyed and created again (after
// cudaDeviceReset the module loads anew and the array can move). The
// lookup allocates nothing.
double* noalloc_workspace()
{
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_ws);
    if (e != cudaSuccess) {
        (void) cudaGetLastError();
        throw mbg::cuda_error(std::string("CUDA: cudaGetSymbolAddress(workspace): ") + cudaGetErrorString(e));
    }
    return static_cast<double*>(p);
}

// Hermitian operator from the qm_operator packing (diagonal, then the upper
// triangle in column-major order as (re, im) pairs)
void fill_op(const double* diag, const double* off, int N, double* re, double* im)
{
    for (int i = 0; i < N * N; i++) re[i] = im[i] = 0.0;
    for (int i = 0; i < N; i++) re[i * N + i] = diag[i];
    for (int k = 1; k < N; k++)
        for (int j = 0; j < k; j++) {
            const int q = mbg::pre::upper_index(j, k);
            re[j * N + k] = off[2 * q];
            im[j * N + k] = off[2 * q + 1];
            re[k * N + j] = off[2 * q];
            im[k * N + j] = -off[2 * q + 1];
        }
}

void fill_mat_in(const mbg_material& mt, int N, double dt, mbg::pre::mat_in& in)
{
    std::memset(&in, 0, sizeof(in));
    in.eps_r = mt.rel_permittivity;
    in.mu_r = mt.rel_permeability;
    in.overlap = mt.overlap_factor;
    in.losses = mt.losses;
    in.dt = dt;
    in.dx = 1.0;
    const mbg_qm& q = *mt.qm;
    in.N = N;
    in.relax_kind = q.relax_kind;
    in.carrier_density = q.carrier_density;
    fill_op(q.h_diag, q.h_off, N, in.h_re, in.h_im);
    fill_op(q.mu_diag, q.mu_off, N, in.mu_re, in.mu_im);
    if (q.relax_kind == MBG_RELAX_LINDBLAD) {
        for (int i = 0; i < N * N; i++) in.S[i] = q.scattering[i];
        for (int i = 0; i < N * (N - 1) / 2; i++) in.deph[i] = q.dephasing[i];
    }
}

}  // namespace

namespace mbg {
void set_last_error(const char* msg);  // capi.cu
}

extern "C" {

int mbg_material_constants_noalloc(
    const char* algo,
    const mbg_material* mat,
    double timestep,
    double* out_device,
    size_t cap,
    size_t* len,
    void* stream)
{
    try {
        if (!algo || !mat || !len) throw mbg::invalid_argument("null argument");
        int kind = std::strcmp(algo, "cvr-rodr") == 0 ? mbg::ALGO_CVR
            : std::strcmp(algo, "reg-cayley") == 0    ? mbg::ALGO_CAYLEY
                                                      : -1;
        if (kind < 0) throw mbg::invalid_argument("algo must be cvr-rodr or reg-cayley");
        if (!mat->qm) throw mbg::invalid_argument("material has no quantum-mechanical description");
        const int N = (int) mat->qm->num_levels;
        if (N < 2 || N > mbg::MAX_LEVELS) throw mbg::invalid_argument("levels must be 2..6");
        const size_t need = kind == mbg::ALGO_CVR ? mbg::pre::cvr_workspace(N) : mbg::pre::cay_workspace(N);
        if (need > NOALLOC_STATUS_SLOT) {
            throw mbg::invalid_argument(
                "workspace of " + std::to_string(need) + " doubles exceeds the fixed " +
                std::to_string(NOALLOC_STATUS_SLOT) + "-double array");
        }
        const int stride = kind == mbg::ALGO_CVR ? mbg::pre::make_cvr_layout(N).stride
                                                 : mbg::pre::make_cay_layout(N).stride;
        *len = (size_t) stride;
        if (!out_device) return MBG_OK;  // size query
        if (cap < (size_t) stride)
            throw mbg::invalid_argument("output buffer holds " + std::to_string(cap) + " doubles, " +
                                        std::to_string(stride) + " needed");
        // the material as the precompute reads it (dx = 1 m, as
        // mbg_material_constants uses); no host or device allocation
        mbg::pre::mat_in in;
        fill_mat_in(*mat, N, timestep, in);
        if (kind == mbg::ALGO_CAYLEY && in.relax_kind != MBG_RELAX_LINDBLAD)
            throw mbg::invalid_argument("Unsupported superoperator!");
        double* ws = noalloc_workspace();
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        precompute_noalloc_kernel<<<1, 1, 0, s>>>(in, kind, N, ws, out_device);
        MBG_CK(cudaGetLastError());
        int code = 0;
        MBG_CK(cudaMemcpyAsync(&code, ws + NOALLOC_STATUS_SLOT, sizeof(int), cudaMemcpyDeviceToHost, s));
        MBG_CK(cudaStreamSynchronize(s));
        if (code == 1) throw mbg::invalid_argument("Number of energy levels does not match selected solver!");
        if (code == 2) throw mbg::invalid_argument("Time-indepent matrix not invertible!");
        if (code == 3) throw mbg::invalid_argument("Unsupported superoperator!");
        if (code != 0) throw std::runtime_error("precompute did not report a status");
        return MBG_OK;
    } catch (const mbg::cuda_error& e) {
        mbg::set_last_error(e.what());
        return MBG_ERR_CUDA;
    } catch (const std::invalid_argument& e) {
        mbg::set_last_error(e.what());
        return MBG_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        mbg::set_last_error(e.what());
        return MBG_ERR_RUNTIME;
    }
}

}  // extern "C"
