// knc_noalloc.cu — primitive recovery that allocates no device memory.
//
// Who needs it: callers that own every byte of device memory themselves and
// cannot let a library call cudaMalloc. Examples are a host that hands the
// whole GPU to its own pool or caching allocator (a cudaMalloc from a library
// could fail or fragment that pool), and a time-critical driver loop where
// cudaMalloc's implicit device synchronisation is not acceptable. The regular
// entry point, knc_get_primitives, needs a context whose buffers are
// allocated with cudaMalloc. This one takes the caller's device buffers for
// input and output.
//
// Its only working memory is the file-scope array below, a fixed 1 MiB plus
// a status word per GPU that loads the library, held until the process
// exits. It holds the block's cell volumes and the first-failure key. The
// volumes are computed on the host (same formulas as every other entry
// point) and copied in at each call; the status word is reset at each call.
//
// Calls share that array and it keeps the last call's contents, so calls
// whose GPU work overlaps (different streams or host threads at the same
// time) race on it: serialise them.
#include <cstdio>
#include <cstring>
#include <vector>

#include "knc_internal.h"
#include "knc_physics.cuh"

namespace knc {

constexpr int64_t NOALLOC_STATUS_OFFSET = KNC_NOALLOC_MAX_ZONES;   // in doubles
constexpr int64_t NOALLOC_SCRATCH_DOUBLES = KNC_NOALLOC_MAX_ZONES + 32;

// Device scratch: [0, MAX_ZONES) cell volumes of the block, then one
// 64-bit first-failure key (zone << 4 | kind, all ones when clean).
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

// Same arithmetic as c2p_f64_kernel<false> followed by prims_to_aos_kernel
// (this file is compiled with the same --fmad=false), so the output equals
// knc_get_primitives' bit for bit.
__global__ void recover_noalloc_kernel(const double* __restrict__ cons, const double* __restrict__ scalar,
                                       double* __restrict__ prim, int64_t n, int32_t srhd, double gm,
                                       double* __restrict__ scratch) {
    const int64_t z = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= n) return;
    const double dV = scratch[z];
    double u[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) u[q] = cons[z * 4 + q] / dV;
    double P[4] = {0.0, 0.0, 0.0, 0.0};
    double bad = 0.0;
    int iters = 0, kind;
    if (srhd) kind = srhd_c2p_newton(gm, u, 0.0, P, iters, bad);
    else kind = newt_c2p(gm - 1.0, u, P, bad);
    if (kind != HYDRO_NONE && kind != HYDRO_NEGATIVE_PRESSURE) {
        unsigned long long* key = reinterpret_cast<unsigned long long*>(scratch + NOALLOC_STATUS_OFFSET);
        atomicMin(key, ((unsigned long long)z << 4) | (unsigned long long)kind);
    }
    const double w = srhd ? sqrt(1.0 + P[1] * P[1] + P[2] * P[2]) : 1.0;
    double v[5] = {P[0], P[1], P[2], P[3], scalar[z] / dV / w};
    v[4] = v[4] / v[0];
#pragma unroll
    for (int q = 0; q < 5; ++q) prim[z * 5 + q] = v[q];
}

namespace {

void fill_error(knc_error* err, int kind, const char* msg) {
    if (!err) return;
    std::memset(err, 0, sizeof(*err));
    err->kind = kind;
    std::snprintf(err->message, sizeof(err->message), "%s", msg);
}

}  // namespace
}  // namespace knc

using namespace knc;

extern "C" int knc_recover_primitives_noalloc(const knc_hydro_params* hydro, const knc_mesh_params* mesh,
                                              int32_t block_index, const double* d_cons, const double* d_scalar,
                                              double* d_prim, void* stream, knc_error* err) {
    if (err) std::memset(err, 0, sizeof(*err));
    if (!hydro || !mesh || !d_cons || !d_scalar || !d_prim) {
        fill_error(err, KNC_HYDRO_NONE, "knc_recover_primitives_noalloc: null argument");
        return KNC_ERR_INVALID_ARGUMENT;
    }
    if (!(hydro->gamma_law_index > 1.0) ||
        (hydro->system != KNC_SYSTEM_RELATIVISTIC && hydro->system != KNC_SYSTEM_NEWTONIAN) ||
        mesh->block_size < 2 || mesh->num_polar_zones < 1 || mesh->reference_radius <= 0.0) {
        fill_error(err, KNC_HYDRO_NONE, "knc_recover_primitives_noalloc: invalid hydro or mesh parameters");
        return KNC_ERR_CONFIG;
    }
    const int64_t nr = mesh->block_size, nq = mesh->num_polar_zones;
    const int64_t n = nr * nq;
    if (n > KNC_NOALLOC_MAX_ZONES) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "knc_recover_primitives_noalloc: a block of %lld zones exceeds the fixed scratch of "
                      "%d zones (KNC_NOALLOC_MAX_ZONES); use knc_get_primitives",
                      (long long)n, (int)KNC_NOALLOC_MAX_ZONES);
        fill_error(err, KNC_HYDRO_NONE, msg);
        return KNC_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

    // The scratch array's name is only a host-side stand-in: resolve its
    // device address on the current device at every call (cheap once the
    // module is loaded), so that no address outlives a device reset.
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        fill_error(err, KNC_HYDRO_NONE, "knc_recover_primitives_noalloc: no current CUDA device");
        return KNC_ERR_CUDA;
    }
    double* scratch = nullptr;
    {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            char msg[256];
            std::snprintf(msg, sizeof(msg), "knc_recover_primitives_noalloc: cudaGetSymbolAddress: %s",
                          cudaGetErrorString(e));
            fill_error(err, KNC_HYDRO_NONE, msg);
            return KNC_ERR_CUDA;
        }
        scratch = static_cast<double*>(p);
    }

    // Cell volumes of the block (src/mesh.rs:119-123, 246-264) into the scratch.
    std::vector<double> dv, rc, qc;
    host_block_volumes(*mesh, block_index, dv, rc, qc);
    cudaError_t e = cudaMemcpyAsync(scratch, dv.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    unsigned long long* d_key = reinterpret_cast<unsigned long long*>(scratch + NOALLOC_STATUS_OFFSET);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_key, 0xff, sizeof(unsigned long long), s);   // "no failure"
    if (e == cudaSuccess) {
        recover_noalloc_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
            d_cons, d_scalar, d_prim, n, hydro->system == KNC_SYSTEM_RELATIVISTIC ? 1 : 0, hydro->gamma_law_index,
            scratch);
        e = cudaGetLastError();
    }
    unsigned long long key = ~0ull;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&key, d_key, sizeof(key), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        char msg[256];
        std::snprintf(msg, sizeof(msg), "knc_recover_primitives_noalloc: %s", cudaGetErrorString(e));
        fill_error(err, KNC_HYDRO_NONE, msg);
        return KNC_ERR_CUDA;
    }
    if (key != ~0ull) {
        const int64_t z = (int64_t)(key >> 4);
        const int kind = (int)(key & 0xf);
        if (err) {
            err->kind = kind;
            err->block = block_index;
            err->i = (int32_t)(z / nq);
            err->j = (int32_t)(z % nq);
            err->r = rc[z / nq];
            err->theta = qc[z % nq];
            double u[4] = {0, 0, 0, 0};
            if (cudaMemcpy(u, d_cons + z * 4, sizeof(u), cudaMemcpyDeviceToHost) == cudaSuccess)
                err->value = (kind == KNC_HYDRO_NEGATIVE_ENERGY_DENSITY ? u[3] : u[0]) / dv[z];
            static const char* names[] = {"None", "NegativeDensity", "NegativePressure", "NegativeEnergyDensity",
                                          "RootFinderFailed"};
            std::snprintf(err->message, sizeof(err->message),
                          "%s(%.4e) at position (r, theta) = (%.4e, %.4f) in block %d zone (%d, %d)",
                          names[kind <= 4 ? kind : 0], err->value, err->r, err->theta, block_index, err->i, err->j);
        }
        return KNC_ERR_HYDRO;
    }
    return KNC_OK;
}
