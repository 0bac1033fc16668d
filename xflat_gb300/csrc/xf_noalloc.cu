// Allocation-free Hamiltonian evaluation (xf_calc_hvv_static).
//
// Some callers of this library cannot call cudaMalloc: host programs whose
// device memory is owned and budgeted up front by another allocator (a
// framework's memory pool, or a fixed reservation made at start-up), and
// per-step loops that must not pay cudaMalloc's implicit device
// synchronisation.  This entry point evaluates phy::calc_Hvv
// (src/Phy_MA.cpp:388-474, src/Phy_MAA.cpp:468-621) on device buffers the
// caller owns and allocates nothing: its scratch (per-beam energy sums, block
// partials of the moment reduction, the last-block ticket and the moments)
// lives in one file-scope device array of fixed size, held by every GPU that
// loads the library until the process exits.
//
// Limits and behaviour:
//  * at most kMaxBeams = 65536 beams (abins * pbins * 4): 2 MiB of per-beam
//    sums plus 64 KiB of block partials; larger inputs are rejected with
//    XF_EINVAL before any work is queued;
//  * the first call on a device looks the array's device address up with
//    cudaGetSymbolAddress (once per device, with that device current); make
//    that first call before any stream capture begins;
//  * every call shares the one array and it keeps the last call's contents:
//    each call clears the ticket it needs at zero, and calls that overlap on
//    the GPU (different streams or threads, without ordering) race on it;
//  * `stream` must belong to the current device (XF_EINVAL otherwise), since
//    the array's address is the current device's;
//  * a CUDA error already pending when the call starts (left by the caller's
//    own work) is reported as XF_ECUDA and left pending for the caller; a
//    launch that fails is reported at once, before the next one is queued.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "xflat_gpu.h"

namespace {

constexpr int kMaxBeams = 65536;
constexpr int kBlocks = 256;       // moment-reduction grid (block partials)
constexpr int kThreads = 256;
constexpr int kSlots = 32;         // doubles per block partial
constexpr size_t kOffS = 0;                                  // [kMaxBeams][4] per-beam sums
constexpr size_t kOffPart = kOffS + (size_t)kMaxBeams * 4;   // [kBlocks][kSlots]
constexpr size_t kOffJ = kOffPart + (size_t)kBlocks * kSlots;  // [16] moments
constexpr size_t kOffTicket = kOffJ + 16;                    // one slot, used as unsigned int
constexpr size_t kScratchDoubles = kOffTicket + 4;

static __device__ __align__(256) double g_hvv_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device (looked up once
// per device).
int scratch_address(double** out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return XF_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return XF_EUNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_hvv_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "xf_calc_hvv_static: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return XF_ECUDA;
        }
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return XF_OK;
}

struct StaticArgs {
    int geom, A, P, ne, epad, nbeams;
    const double* psi;
    const double* fv;
    const double* cosb;
    const double* sinb;
    const double* dcosb;
    const double* cosphi;
    const double* sinphi;
    double LE[4];
    double kappa;
    double* scratch;
    double* hvv;
};

__device__ __forceinline__ int comp_of(int i) { return i == 0 ? 0 : (i == 1 ? 2 : 3); }

// NBeam::calcESum (src/NBeam.cpp:812-840): one warp per beam, lanes over energies.
__global__ void k_static_esum(StaticArgs a)
{
    const int lane = threadIdx.x & 31;
    const int warps = blockDim.x >> 5;
    double* S = a.scratch + kOffS;
    for (int b = blockIdx.x * warps + (threadIdx.x >> 5); b < a.nbeams; b += gridDim.x * warps) {
        const double* x = a.psi + (size_t)b * 4 * a.epad;
        const double* fv = a.fv + (size_t)(b & 3) * a.epad;
        double s0 = 0., s2 = 0., s3 = 0.;
        for (int e = lane; e < a.ne; e += 32) {
            const double ar = x[e], ai = x[a.epad + e], br = x[2 * a.epad + e], bi = x[3 * a.epad + e];
            const double f = fv[e];
            s0 = fma((ar * ar + ai * ai) - (br * br + bi * bi), f, s0);
            s2 = fma(ar * br + ai * bi, f, s2);
            s3 = fma(ai * br - ar * bi, f, s3);
        }
        for (int off = 16; off >= 1; off >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, off);
            s2 += __shfl_xor_sync(0xffffffffu, s2, off);
            s3 += __shfl_xor_sync(0xffffffffu, s3, off);
        }
        if (lane == 0) {
            S[(size_t)b * 4 + 0] = .5 * s0;
            S[(size_t)b * 4 + 1] = 0.;
            S[(size_t)b * 4 + 2] = s2;
            S[(size_t)b * 4 + 3] = s3;
        }
    }
}

// Angular moments from the per-beam sums (the flavor combination of
// include/NBeam.h:47-53 and the angle weights of src/Phy_MA.cpp:418-426 /
// src/Phy_MAA.cpp:513-536); one thread per beam, block partials in the
// scratch array, the last block to finish sums them in block order.
__global__ void k_static_moments(StaticArgs a)
{
    __shared__ double sh[kThreads][12];
    __shared__ int is_last;
    const int K = a.geom == 0 ? 2 : 4;
    double acc[12];
    for (int i = 0; i < 12; ++i) acc[i] = 0.;
    const double* S = a.scratch + kOffS;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < a.nbeams; b += gridDim.x * blockDim.x) {
        const int p = b & 3, ap = b >> 2, ang = ap / a.P, phi = ap - ang * a.P;
        const double dc = a.dcosb[ang], c = a.cosb[ang];
        for (int i = 0; i < 3; ++i) {
            const int z = comp_of(i);
            const double sgn = (z == 3 || (p & 1) == 0) ? 1.0 : -1.0;
            const double w = (S[(size_t)b * 4 + z] * a.LE[p]) * sgn;
            acc[i * K + 0] += w * dc;
            if (a.geom == 0) {
                acc[i * K + 1] += w * dc * c;
            } else {
                const double s = a.sinb[ang];
                acc[i * K + 1] += w * a.cosphi[phi] * s * dc;
                acc[i * K + 2] += w * a.sinphi[phi] * s * dc;
                acc[i * K + 3] += w * dc * c;
            }
        }
    }
    for (int i = 0; i < 12; ++i) sh[threadIdx.x][i] = acc[i];
    __syncthreads();
    for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
        if ((int)threadIdx.x < stride)
            for (int i = 0; i < 12; ++i) sh[threadIdx.x][i] += sh[threadIdx.x + stride][i];
        __syncthreads();
    }
    double* part = a.scratch + kOffPart + (size_t)blockIdx.x * kSlots;
    if (threadIdx.x < 12) part[threadIdx.x] = sh[0][threadIdx.x];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int* ticket = reinterpret_cast<unsigned int*>(a.scratch + kOffTicket);
        is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double* J = a.scratch + kOffJ;
    if (threadIdx.x < 16) J[threadIdx.x] = 0.;
    __syncthreads();
    if ((int)threadIdx.x < 3 * K) {
        double t = 0.;
        for (unsigned blk = 0; blk < gridDim.x; ++blk) t += __ldcg(a.scratch + kOffPart + (size_t)blk * kSlots + threadIdx.x);
        const int i = threadIdx.x / K, k = threadIdx.x % K;
        J[k * 4 + comp_of(i)] = t;
    }
}

// phy::getHvv for every (theta, phi) bin (src/Phy_MA.cpp:372-377, src/Phy_MAA.cpp:445-461).
__global__ void k_static_hvv(StaticArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.A * a.P) return;
    const int ang = i / a.P, phi = i - ang * a.P;
    const double* J = a.scratch + kOffJ;
    const double c = a.cosb[ang];
    for (int z = 0; z < 4; ++z) {
        double h;
        if (a.geom == 0) {
            h = (J[z] - (J[4 + z] * c)) * a.kappa;
        } else {
            const double s = a.sinb[ang], cp = a.cosphi[phi], sp = a.sinphi[phi];
            h = (J[z] - (s * cp * J[4 + z] + s * sp * J[8 + z] + c * J[12 + z])) * a.kappa;
        }
        a.hvv[4 * (size_t)i + z] = h;
    }
}

}  // namespace

extern "C" int xf_calc_hvv_static(int geometry, int abins, int pbins, int ebins, int epad, const double* psi,
                                  const double* fv, const double* cosb, const double* sinb, const double* dcosb,
                                  const double* cosphi, const double* sinphi, const double* LE, double kappa,
                                  double* hvv, void* stream)
{
    if (geometry != XF_GEOM_MA && geometry != XF_GEOM_MAA) return XF_EINVAL;
    const int P = geometry == XF_GEOM_MAA ? pbins : 1;
    if (abins <= 0 || P <= 0 || ebins <= 0 || epad < ebins) return XF_EINVAL;
    const long long nbeams = (long long)abins * P * 4;
    if (nbeams > kMaxBeams) {
        std::fprintf(stderr,
                     "xf_calc_hvv_static: %lld beams exceed the static scratch limit of %d beams "
                     "(abins * pbins * 4); use xf_calc_hvv instead\n", nbeams, kMaxBeams);
        return XF_EINVAL;
    }
    if (!psi || !fv || !cosb || !dcosb || !LE || !hvv) return XF_EINVAL;
    if (geometry == XF_GEOM_MAA && (!sinb || !cosphi || !sinphi)) return XF_EINVAL;
    // an error left by earlier work stays the caller's to see
    if (cudaPeekAtLastError() != cudaSuccess) return XF_ECUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int cur = -1, sdev = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) return XF_ECUDA;
    if (st) {
        if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) return XF_EINVAL;
        if (sdev != cur) {
            std::fprintf(stderr, "xf_calc_hvv_static: the stream belongs to device %d, the current device is %d\n",
                         sdev, cur);
            return XF_EINVAL;
        }
    }
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    StaticArgs a;
    a.geom = geometry;
    a.A = abins;
    a.P = P;
    a.ne = ebins;
    a.epad = epad;
    a.nbeams = (int)nbeams;
    a.psi = psi;
    a.fv = fv;
    a.cosb = cosb;
    a.sinb = sinb;
    a.dcosb = dcosb;
    a.cosphi = cosphi;
    a.sinphi = sinphi;
    for (int p = 0; p < 4; ++p) a.LE[p] = LE[p];
    a.kappa = kappa;
    a.scratch = scratch;
    a.hvv = hvv;
    // the ticket of the last-block reduction must start at zero on every call
    if (cudaMemsetAsync(scratch + kOffTicket, 0, sizeof(unsigned int), st) != cudaSuccess) return XF_ECUDA;
    const int warps = kThreads / 32;
    int eb = (int)((nbeams + warps - 1) / warps);
    if (eb > 4096) eb = 4096;
    k_static_esum<<<eb, kThreads, 0, st>>>(a);
    if (cudaGetLastError() != cudaSuccess) return XF_ECUDA;
    int mb = (int)((nbeams + kThreads - 1) / kThreads);
    if (mb > kBlocks) mb = kBlocks;
    k_static_moments<<<mb, kThreads, 0, st>>>(a);
    if (cudaGetLastError() != cudaSuccess) return XF_ECUDA;
    const int nh = abins * P;
    k_static_hvv<<<(nh + 127) / 128, 128, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? XF_OK : XF_ECUDA;
}
