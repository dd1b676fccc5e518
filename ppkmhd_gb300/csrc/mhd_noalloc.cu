// mhd_step_noalloc: one MUSCL-Hancock + HLLD + CT iteration that allocates
// nothing on the device or the host.
//
// Some callers cannot call cudaMalloc: a host application that owns all
// device memory through its own pool and forbids libraries from allocating,
// a latency-bounded loop where an allocation may stall or fail mid-run, or a
// job on a shared GPU that must keep a fixed memory footprint after start-up.
// For them this entry point takes the caller's device arrays for the state
// (input and output) and keeps every intermediate (primitives, slopes,
// half-step state, edge field, face fluxes, edge EMFs and the time-step
// record) in one file-scope __device__ array of MHD_NOALLOC_SCRATCH_BYTES,
// reserved by every GPU that loads this library until the process exits.
//
// The array is shared by all calls and keeps the last call's contents, so
// each call clears the part it uses (cudaMemsetAsync on the caller's stream,
// which allocates nothing) before its kernels run: the halo planes that no
// stage writes (the last plane of the primitives, read by the slopes of the
// last trace plane) then read zeros, as in the context path, whatever grid
// or precision the previous call ran.  Calls that overlap on the GPU
// (concurrent streams, or several host threads) race on the array: serialise
// them.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (host code cannot use the array's name as an address)
// and caches it per device; make that first call before any stream capture.
// A cudaDeviceReset unloads the module and the cached address goes stale:
// calls made after a reset of the device are not supported.
#include <climits>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#define MHD_VARIANT_TAG v_na
#include "mhd_core.h"
#include "mhd_kernels.cuh"
#include "ppkmhd_gb300.h"

// The scratch array itself (device memory; in host code this name is a
// host-side stand-in, never a device address).
static __device__ __align__(256) unsigned char g_noalloc_scratch[MHD_NOALLOC_SCRATCH_BYTES];

namespace
{

using namespace mhd::v_na;

constexpr int kMaxDevices = 64;
std::mutex    g_mutex;
void *        g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once per
// device, with that device current).
int
scratch_address(void ** out, std::string & err)
{
  int         dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
  {
    err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return MHD_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= kMaxDevices)
  {
    err = "device ordinal beyond the no-allocation path's table";
    return MHD_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev])
  {
    void * ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
    {
      err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return MHD_ERR_CUDA;
    }
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return MHD_OK;
}

__global__ void
k_noalloc_reset(DevState * st, double t, double tEnd)
{
  st->t = t;
  st->dt = 0.0;
  st->tEnd = tEnd;
  st->dtdx = st->dtdy = st->dtdz = 0.0;
  st->invdt_bits = 0ull;
  st->it = 0;
  st->nStepmax = 1;
  st->status = 0;
  st->pad = 0;
}

size_t
align256(size_t b)
{
  return (b + 255) & ~(size_t)255;
}

template <class R>
int
step(const mhd_params & p, void * U_in, void * U_out, double t, double * dt, cudaStream_t s,
     std::string & err)
{
  const Grid<R> G = make_grid<R>(p);

  const int     dim = p.dim;
  const size_t  n = (size_t)G.sv;
  const int     ne = dim == 3 ? 3 : 1;
  const int     nf = dim == 3 ? 5 : 6;
  const size_t  b8 = align256(n * NV * sizeof(R));
  const size_t  need = 2 * b8 + align256(n * NV * dim * sizeof(R)) +
                      2 * align256(n * ne * sizeof(R)) + align256(n * nf * dim * sizeof(R)) +
                      align256(n * face_data_planes(dim) * sizeof(R)) + align256(sizeof(DevState));
  if (need > (size_t)MHD_NOALLOC_SCRATCH_BYTES)
  {
    err = "grid needs " + std::to_string(need) + " bytes of scratch; the no-allocation path has " +
          std::to_string((size_t)MHD_NOALLOC_SCRATCH_BYTES);
    return MHD_ERR_TOO_LARGE;
  }
  void * base = nullptr;
  if (int rc = scratch_address(&base, err))
    return rc;
  unsigned char * q = static_cast<unsigned char *>(base);
  Buffers<R>      B{};
  B.Uin = static_cast<R *>(U_in);
  B.Uout = static_cast<R *>(U_out);
  B.Q = reinterpret_cast<R *>(q);
  q += b8;
  B.Q2 = reinterpret_cast<R *>(q);
  q += b8;
  B.S = reinterpret_cast<R *>(q);
  q += align256(n * NV * dim * sizeof(R));
  B.E = reinterpret_cast<R *>(q);
  q += align256(n * ne * sizeof(R));
  B.F = reinterpret_cast<R *>(q);
  q += align256(n * nf * dim * sizeof(R));
  B.Em = reinterpret_cast<R *>(q);
  q += align256(n * ne * sizeof(R));
  B.H = reinterpret_cast<R *>(q);
  q += align256(n * face_data_planes(dim) * sizeof(R));
  B.st = reinterpret_cast<DevState *>(q);

  auto nb = [](int64_t cnt, int th) { return (unsigned)((cnt + th - 1) / th); };
  cudaError_t e = cudaMemsetAsync(base, 0, need, s);
  if (e != cudaSuccess)
  {
    err = std::string("clearing the scratch array: ") + cudaGetErrorString(e);
    return MHD_ERR_CUDA;
  }
  k_noalloc_reset<<<1, 1, 0, s>>>(B.st, t, p.tEnd);
  const int64_t nprim = (int64_t)(G.isize - 1) * (G.jsize - 1) * (dim == 3 ? G.ksize - 1 : 1);
  const int64_t ntrace = (int64_t)(G.nx + 3) * (G.ny + 3) * (dim == 3 ? G.nz + 3 : 1);
  const int64_t nface = (int64_t)(G.nx + 1) * (G.ny + 1) * (dim == 3 ? G.nz + 1 : 1);
  const int64_t ncell = (int64_t)G.nx * G.ny * (dim == 3 ? G.nz : 1);
  if (dim == 2)
  {
    k_boundaries<R, 2><<<nb(ghost_count<R, 2>(G), 256), 256, 0, s>>>(G, B.Uin, B.st, 0);
    k_prim_dt<R, 2><<<nb(nprim, 256), 256, 0, s>>>(G, B.Uin, B.Q, B.st, 0);
    k_finalize_dt<R><<<1, 1, 0, s>>>(G, B.st, 0);
    k_trace<R, 2><<<nb(ntrace, 128), 128, 0, s>>>(G, B);
    k_flux<R, 2><<<dim3(nb(nface, 128), 2), 128, 0, s>>>(G, B);
    k_emf<R, 2><<<dim3(nb(nface, 128), 1), 128, 0, s>>>(G, B, 0, nface);
    k_update<R, 2><<<nb(ncell, 256), 256, 0, s>>>(G, B, 0, ncell);
  }
  else
  {
    k_boundaries<R, 3><<<nb(ghost_count<R, 3>(G), 256), 256, 0, s>>>(G, B.Uin, B.st, 0);
    k_prim_dt<R, 3><<<nb(nprim, 256), 256, 0, s>>>(G, B.Uin, B.Q, B.st, 0);
    k_finalize_dt<R><<<1, 1, 0, s>>>(G, B.st, 0);
    k_trace<R, 3><<<nb(ntrace, 128), 128, 0, s>>>(G, B);
    k_flux<R, 3><<<dim3(nb(nface, 128), 3), 128, 0, s>>>(G, B);
    k_emf<R, 3><<<dim3(nb(nface, 128), 3), 128, 0, s>>>(G, B, 0, nface);
    k_update<R, 3><<<nb(ncell, 256), 256, 0, s>>>(G, B, 0, ncell);
  }
  k_advance<R><<<1, 1, 0, s>>>(B.st);
  e = cudaGetLastError();
  if (e != cudaSuccess)
  {
    err = std::string("kernel launch: ") + cudaGetErrorString(e);
    return MHD_ERR_CUDA;
  }
  DevState h{};
  e = cudaMemcpyAsync(&h, B.st, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
  {
    err = std::string("reading the time-step record: ") + cudaGetErrorString(e);
    return MHD_ERR_CUDA;
  }
  *dt = h.it == 1 ? h.dt : 0.0;
  if (h.status & STATUS_NUMERIC)
  {
    err = "non-finite or non-positive state detected (density, energy or CFL rate)";
    return MHD_ERR_NUMERIC;
  }
  return MHD_OK;
}

} // namespace

extern "C"
{

  int
  mhd_step_noalloc(const mhd_params * p, void * U_in, void * U_out, double t, double * dt,
                   void * stream)
  {
    if (!p || !U_in || !U_out || !dt || U_in == U_out)
      return MHD_ERR_INVALID_ARG;
    if (!mhd::validate_params(*p).empty() || p->solver != MHD_SOLVER_MHD_MUSCL ||
        p->fp_mode != MHD_FP_FAST || p->implementation_version != 2)
      return MHD_ERR_INVALID_ARG;
    // the reference's finished() test (SolverBase.cpp:195-201): nothing to do
    if (t >= p->tEnd - 1e-14)
    {
      *dt = 0.0;
      return MHD_FINISHED;
    }
    // run on p->device and give the caller's current device back afterwards
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess)
      return MHD_ERR_NO_DEVICE;
    if (prev != p->device && cudaSetDevice(p->device) != cudaSuccess)
      return MHD_ERR_NO_DEVICE;
    std::string  err; // status codes carry the outcome; the text is not kept
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int    rc = p->precision == MHD_FP32 ? step<float>(*p, U_in, U_out, t, dt, s, err)
                                               : step<double>(*p, U_in, U_out, t, dt, s, err);
    if (prev != p->device)
      cudaSetDevice(prev);
    return rc;
  }

} // extern "C"
