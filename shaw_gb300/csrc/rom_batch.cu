// rom_batch.cu -- a batch of independent rank-2 reduced systems of uneven size (their own
// kv, ks and forcing count M) advanced together.
//
// Every instance is the reduced system of runRomRankTwoForcing
// (src/kokkos/torevise/run_rom_rank_two_forcing.hpp:149-188):
//   XV += dt Av XS ;  XV[:,j] += (f_j(t_{n-1}) dt) b[:,j] ;  XS += dt As XV
// The reference runs one system per process; a batch has no counterpart there.
//   SHAW_FP64              per step: one cuBLAS DGEMM per instance for each half-step and
//                          ONE forcing kernel over the columns of all instances;
//   SHAW_MIXED_OZAKI_BF16  the whole run of every instance in ONE persistent tensor-core
//                          launch (rom_oz.cu), tile widths and schedule from the autotuner.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "rom_oz.h"
#include "shaw_internal.h"

namespace {

struct BInst {
  uint64_t kv = 0, ks = 0;
  uint32_t M = 0;
  double *Av = nullptr, *As = nullptr, *b = nullptr, *xv = nullptr, *xs = nullptr;  // FP64 path
  int* kind = nullptr;
  double *period = nullptr, *delay = nullptr;
  // reduced-state snapshots (device, k x T x M) and the caller's host arrays
  uint64_t fvp = 0, fsp = 0, snap_nsteps = 0;
  double *snap_vp = nullptr, *snap_sp = nullptr, *host_vp = nullptr, *host_sp = nullptr;
  // receivers: rows PhiVp[gid_r, :] (device, FP64 path) and the seismogram R x T x M (device)
  uint32_t R = 0;
  uint64_t fseis = 0, seis_T = 0, seis_nsteps = 0;
  double *phi_rcv = nullptr, *seis = nullptr;
};

// Column c of the batch (over all instances) -> its instance data, for the FP64 forcing kernel.
struct ColRef {
  double* xv;
  const double* b;
  const int* kind;
  const double* period;
  const double* delay;
  uint32_t kv, j;
};

// XV[:, j] += (f_j(t_{n-1}) dt) b[:, j] for every column of every instance (one block per column).
__global__ void rom_batch_forcing_kernel(const ColRef* cols, double dt, unsigned long long n) {
  __shared__ double fdt;
  const ColRef c = cols[blockIdx.x];
  if (threadIdx.x == 0) fdt = shaw::signal_value(c.kind[c.j], c.delay[c.j], c.period[c.j], (double)(n - 1) * dt) * dt;
  __syncthreads();
  double* x = c.xv + (size_t)c.j * c.kv;
  const double* bc = c.b + (size_t)c.j * c.kv;
  for (uint32_t i = threadIdx.x; i < c.kv; i += blockDim.x) x[i] = __dadd_rn(x[i], __dmul_rn(fdt, bc[i]));
}

}  // namespace

struct shaw_rom_batch_s {
  int precision = SHAW_FP64;
  cudaStream_t stream = nullptr;
  cublasHandle_t blas = nullptr;
  std::vector<BInst> inst;
  ColRef* cols = nullptr;
  uint64_t ncols = 0;
  shaw::oz::Batch* oz = nullptr;
  uint64_t step = 0, launches = 0;
};

namespace {

using BH = shaw_rom_batch_s;

int fp64_step(BH* h, double dt, uint64_t n) {
  const double one = 1.0;
  for (BInst& in : h->inst) {
    // xv = xv + dt * Av xs  (Av row-major kv x ks == column-major ks x kv -> op T)
    if (cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)in.kv, (int)in.M, (int)in.ks, &dt, in.Av, (int)in.ks,
                    in.xs, (int)in.ks, &one, in.xv, (int)in.kv) != CUBLAS_STATUS_SUCCESS)
      return shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (velocity) failed");
  }
  rom_batch_forcing_kernel<<<(unsigned)h->ncols, 128, 0, h->stream>>>(h->cols, dt, n);
  SHAW_CUDA(cudaGetLastError());
  h->launches += h->inst.size() + 1;
  for (BInst& in : h->inst) {
    if (in.fseis && n % in.fseis == 0) {
      // S(:, t, :) = PhiRcv (R x kv) XV (kv x M)  (main_reconstruct_seismo.cc:157-185)
      const double one1 = 1.0, zero = 0.0;
      if (cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)in.R, (int)in.M, (int)in.kv, &one1, in.phi_rcv,
                      (int)in.kv, in.xv, (int)in.kv, &zero, in.seis + (size_t)in.R * (n / in.fseis - 1),
                      (int)(in.R * in.seis_T)) != CUBLAS_STATUS_SUCCESS)
        return shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (seismogram) failed");
      h->launches++;
    }
    if (in.fvp && n % in.fvp == 0) {
      const uint64_t T = in.snap_nsteps / in.fvp;
      SHAW_CUDA(cudaMemcpy2DAsync(in.snap_vp + in.kv * (n / in.fvp - 1), in.kv * T * sizeof(double), in.xv,
                                  in.kv * sizeof(double), in.kv * sizeof(double), in.M, cudaMemcpyDeviceToDevice,
                                  h->stream));
    }
    // xs = xs + dt * As xv
    if (cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)in.ks, (int)in.M, (int)in.kv, &dt, in.As, (int)in.kv,
                    in.xv, (int)in.kv, &one, in.xs, (int)in.ks) != CUBLAS_STATUS_SUCCESS)
      return shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (stress) failed");
    h->launches++;
    if (in.fsp && n % in.fsp == 0) {
      const uint64_t T = in.snap_nsteps / in.fsp;
      SHAW_CUDA(cudaMemcpy2DAsync(in.snap_sp + in.ks * (n / in.fsp - 1), in.ks * T * sizeof(double), in.xs,
                                  in.ks * sizeof(double), in.ks * sizeof(double), in.M, cudaMemcpyDeviceToDevice,
                                  h->stream));
    }
  }
  return SHAW_OK;
}

}  // namespace

extern "C" {

void shaw_rom_batch_destroy(shaw_rom_batch_t h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->oz) shaw::oz::destroy(h->oz);
  for (BInst& in : h->inst) {
    void* bufs[] = {in.Av, in.As, in.b, in.xv, in.xs, in.kind, in.period, in.delay, in.snap_vp, in.snap_sp,
                    in.phi_rcv, in.seis};
    for (void* p : bufs)
      if (p) cudaFree(p);
  }
  if (h->cols) cudaFree(h->cols);
  if (h->blas) cublasDestroy(h->blas);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int shaw_rom_batch_create(uint32_t n, const shaw_rom_instance_desc* desc, int precision, shaw_rom_batch_t* out) {
  if (!out || !desc) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (n == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "a batch needs at least one instance");
  if (precision != SHAW_FP64 && precision != SHAW_MIXED_OZAKI_BF16 && precision != SHAW_OZAKI_FP64)
    return shaw::fail(SHAW_ERR_UNSUPPORTED,
                      "batched ROM precision must be SHAW_FP64, SHAW_MIXED_OZAKI_BF16 or SHAW_OZAKI_FP64");
  for (uint32_t i = 0; i < n; ++i) {
    const shaw_rom_instance_desc& d = desc[i];
    const std::string who = "instance " + std::to_string(i) + ": ";
    if (!d.rom_jvp || !d.rom_jsp || !d.b || !d.kind || !d.period || !d.delay)
      return shaw::fail(SHAW_ERR_INVALID_ARG, who + "null array");
    if (d.kv == 0 || d.ks == 0 || d.num_forcings == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, who + "empty sizes");
    if (d.kv > 65535 || d.ks > 65535) return shaw::fail(SHAW_ERR_UNSUPPORTED, who + "at most 65535 modes");
    for (uint32_t j = 0; j < d.num_forcings; ++j) {
      if (d.kind[j] < SHAW_SIGNAL_RICKER || d.kind[j] > SHAW_SIGNAL_GAUSS_DER)
        return shaw::fail(SHAW_ERR_INVALID_ARG, who + "unknown signal kind");
      if (!(d.period[j] > 0.0)) return shaw::fail(SHAW_ERR_INVALID_ARG, who + "Period for signal must be positive. ");
      if (!(d.delay[j] >= 0.0)) return shaw::fail(SHAW_ERR_INVALID_ARG, who + "Delay time of the signal must be >=0");
    }
  }
  BH* h = new BH();
  h->precision = precision;
  auto bail = [&](int rc) {
    shaw_rom_batch_destroy(h);
    return rc;
  };
  cudaError_t e;
#define SHAW_TRY(call) do { e = (call); if (e != cudaSuccess) return bail(shaw::cuda_fail(e, #call)); } while (0)
  SHAW_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  h->inst.resize(n);
  std::vector<ColRef> cols;
  for (uint32_t i = 0; i < n; ++i) {
    const shaw_rom_instance_desc& d = desc[i];
    BInst& in = h->inst[i];
    in.kv = d.kv; in.ks = d.ks; in.M = d.num_forcings;
    SHAW_TRY(cudaMalloc(&in.kind, in.M * sizeof(int)));
    SHAW_TRY(cudaMalloc(&in.period, in.M * sizeof(double)));
    SHAW_TRY(cudaMalloc(&in.delay, in.M * sizeof(double)));
    SHAW_TRY(cudaMemcpyAsync(in.kind, d.kind, in.M * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    SHAW_TRY(cudaMemcpyAsync(in.period, d.period, in.M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    SHAW_TRY(cudaMemcpyAsync(in.delay, d.delay, in.M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (precision == SHAW_FP64) {
      SHAW_TRY(cudaMalloc(&in.Av, in.kv * in.ks * sizeof(double)));
      SHAW_TRY(cudaMalloc(&in.As, in.kv * in.ks * sizeof(double)));
      SHAW_TRY(cudaMalloc(&in.b, in.kv * in.M * sizeof(double)));
      SHAW_TRY(cudaMalloc(&in.xv, in.kv * in.M * sizeof(double)));
      SHAW_TRY(cudaMalloc(&in.xs, in.ks * in.M * sizeof(double)));
      SHAW_TRY(cudaMemcpyAsync(in.Av, d.rom_jvp, in.kv * in.ks * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      SHAW_TRY(cudaMemcpyAsync(in.As, d.rom_jsp, in.kv * in.ks * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      SHAW_TRY(cudaMemcpyAsync(in.b, d.b, in.kv * in.M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      for (uint32_t j = 0; j < in.M; ++j) cols.push_back({in.xv, in.b, in.kind, in.period, in.delay, (uint32_t)in.kv, j});
    }
    SHAW_TRY(cudaStreamSynchronize(h->stream));
  }
  if (precision == SHAW_FP64) {
    h->ncols = cols.size();
    SHAW_TRY(cudaMalloc(&h->cols, cols.size() * sizeof(ColRef)));
    SHAW_TRY(cudaMemcpyAsync(h->cols, cols.data(), cols.size() * sizeof(ColRef), cudaMemcpyHostToDevice, h->stream));
    SHAW_TRY(cudaStreamSynchronize(h->stream));
    if (cublasCreate(&h->blas) != CUBLAS_STATUS_SUCCESS) return bail(shaw::fail(SHAW_ERR_CUDA, "cublasCreate failed"));
    if (cublasSetStream(h->blas, h->stream) != CUBLAS_STATUS_SUCCESS)
      return bail(shaw::fail(SHAW_ERR_CUDA, "cublasSetStream failed"));
  } else {
    std::vector<shaw::oz::InstanceDesc> od(n);
    for (uint32_t i = 0; i < n; ++i) {
      od[i].kv = (uint32_t)desc[i].kv; od[i].ks = (uint32_t)desc[i].ks; od[i].M = desc[i].num_forcings;
      od[i].Av = desc[i].rom_jvp; od[i].As = desc[i].rom_jsp; od[i].b = desc[i].b;
    }
    int rc = shaw::oz::create(h->oz, n, od.data(), h->stream, precision == SHAW_OZAKI_FP64 ? 9 : 6);
    for (uint32_t i = 0; rc == SHAW_OK && i < n; ++i)
      rc = shaw::oz::set_signals(h->oz, i, h->inst[i].kind, h->inst[i].period, h->inst[i].delay);
    if (rc) return bail(rc);
    SHAW_TRY(cudaStreamSynchronize(h->stream));
  }
#undef SHAW_TRY
  if (int rc = shaw_rom_batch_reset(h)) return bail(rc);
  *out = h;
  return SHAW_OK;
}

int shaw_rom_batch_reset(shaw_rom_batch_t h) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  h->step = 0;
  if (h->oz) {
    if (int rc = shaw::oz::reset(h->oz, h->stream)) return rc;
  } else {
    for (BInst& in : h->inst) {
      SHAW_CUDA(cudaMemsetAsync(in.xv, 0, in.kv * in.M * sizeof(double), h->stream));
      SHAW_CUDA(cudaMemsetAsync(in.xs, 0, in.ks * in.M * sizeof(double), h->stream));
    }
  }
  for (BInst& in : h->inst) {
    if (in.seis) SHAW_CUDA(cudaMemsetAsync(in.seis, 0, (size_t)in.R * in.seis_T * in.M * 8, h->stream));
    if (in.snap_vp) SHAW_CUDA(cudaMemsetAsync(in.snap_vp, 0, in.kv * (in.snap_nsteps / in.fvp) * in.M * 8, h->stream));
    if (in.snap_sp) SHAW_CUDA(cudaMemsetAsync(in.snap_sp, 0, in.ks * (in.snap_nsteps / in.fsp) * in.M * 8, h->stream));
  }
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  return SHAW_OK;
}

int shaw_rom_batch_set_snapshots(shaw_rom_batch_t h, uint32_t i, uint64_t fvp, uint64_t fsp, uint64_t nsteps,
                                 double* host_vp, double* host_sp) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (i >= h->inst.size()) return shaw::fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  BInst& in = h->inst[i];
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (in.snap_vp) { cudaFree(in.snap_vp); in.snap_vp = nullptr; }
  if (in.snap_sp) { cudaFree(in.snap_sp); in.snap_sp = nullptr; }
  in.fvp = in.fsp = in.snap_nsteps = 0;
  in.host_vp = in.host_sp = nullptr;
  if (fvp == 0 && fsp == 0) {
    if (h->oz) return shaw::oz::set_snapshots(h->oz, i, nullptr, nullptr, 0, 0, 0, 0);
    return SHAW_OK;
  }
  if (fvp == 0 || fsp == 0 || !host_vp || !host_sp)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "snapshot frequencies must be positive and arrays non-null");
  const uint64_t Tv = nsteps / fvp, Ts = nsteps / fsp;
  SHAW_CUDA(cudaMalloc(&in.snap_vp, std::max<uint64_t>(1, in.kv * Tv * in.M) * sizeof(double)));
  SHAW_CUDA(cudaMalloc(&in.snap_sp, std::max<uint64_t>(1, in.ks * Ts * in.M) * sizeof(double)));
  SHAW_CUDA(cudaMemsetAsync(in.snap_vp, 0, in.kv * Tv * in.M * sizeof(double), h->stream));
  SHAW_CUDA(cudaMemsetAsync(in.snap_sp, 0, in.ks * Ts * in.M * sizeof(double), h->stream));
  in.fvp = fvp; in.fsp = fsp; in.snap_nsteps = nsteps; in.host_vp = host_vp; in.host_sp = host_sp;
  if (h->oz) return shaw::oz::set_snapshots(h->oz, i, in.snap_vp, in.snap_sp, Tv, Ts, (uint32_t)fvp, (uint32_t)fsp);
  return SHAW_OK;
}

int shaw_rom_batch_set_receivers(shaw_rom_batch_t h, uint32_t i, const double* phi_rows, uint32_t R, uint64_t freq,
                                 uint64_t nsteps) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (i >= h->inst.size()) return shaw::fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  BInst& in = h->inst[i];
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (in.phi_rcv) { cudaFree(in.phi_rcv); in.phi_rcv = nullptr; }
  if (in.seis) { cudaFree(in.seis); in.seis = nullptr; }
  in.R = 0; in.fseis = in.seis_T = in.seis_nsteps = 0;
  if (h->oz)
    if (int rc = shaw::oz::set_receivers(h->oz, i, nullptr, 0, nullptr, 0, 0, h->stream)) return rc;
  if (R == 0) return SHAW_OK;
  if (!phi_rows) return shaw::fail(SHAW_ERR_INVALID_ARG, "null receiver rows");
  if (freq == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "cannot have seismoFreq <=0 ");
  if (nsteps % freq) return shaw::fail(SHAW_ERR_FREQ_DIVISOR, "Seismogram sampling frequency not a divisor of steps");
  if (freq > 0xFFFFFFFFull) return shaw::fail(SHAW_ERR_UNSUPPORTED, "seismogram frequency too large");
  const uint64_t T = nsteps / freq;
  SHAW_CUDA(cudaMalloc(&in.seis, std::max<size_t>(1, (size_t)R * T * in.M) * sizeof(double)));
  SHAW_CUDA(cudaMemsetAsync(in.seis, 0, (size_t)R * T * in.M * sizeof(double), h->stream));
  if (h->oz) {
    if (int rc = shaw::oz::set_receivers(h->oz, i, phi_rows, R, in.seis, T, (uint32_t)freq, h->stream)) return rc;
  } else {
    SHAW_CUDA(cudaMalloc(&in.phi_rcv, (size_t)R * in.kv * sizeof(double)));
    SHAW_CUDA(cudaMemcpyAsync(in.phi_rcv, phi_rows, (size_t)R * in.kv * sizeof(double), cudaMemcpyHostToDevice,
                              h->stream));
  }
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  in.R = R; in.fseis = freq; in.seis_T = T; in.seis_nsteps = nsteps;
  return SHAW_OK;
}

int shaw_rom_batch_get_seismogram(shaw_rom_batch_t h, uint32_t i, double* out) {
  if (!h || !out) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (i >= h->inst.size()) return shaw::fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  const BInst& in = h->inst[i];
  if (!in.seis) return shaw::fail(SHAW_ERR_STATE, "no receivers set");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  SHAW_CUDA(cudaMemcpy(out, in.seis, (size_t)in.R * in.seis_T * in.M * sizeof(double), cudaMemcpyDeviceToHost));
  return SHAW_OK;
}

int shaw_rom_batch_tune(shaw_rom_batch_t h, double dt, uint64_t trial_steps, char* report, size_t cap) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (!(dt > 0.0) || !std::isfinite(dt)) return shaw::fail(SHAW_ERR_INVALID_ARG, "dt must be > 0");
  std::string rep;
  if (h->oz) {
    unsigned long long n = 0;
    const int rc = shaw::oz::tune(h->oz, h->stream, dt, trial_steps, rep, n);
    h->launches += n;
    if (rc) return rc;
  } else {
    rep = "FP64: cuBLAS DGEMM per instance, nothing to tune\n";
  }
  h->step = 0;
  if (int rc = shaw_rom_batch_reset(h)) return rc;
  if (report && cap) {
    std::strncpy(report, rep.c_str(), cap - 1);
    report[cap - 1] = '\0';
  }
  return SHAW_OK;
}

int shaw_selftest_bounded_waits(uint64_t polls, uint32_t* status) {
  if (!status || polls == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "status must be non-null and polls > 0");
  // the kernels' own limit: a larger count would let the self-test spin far longer
  // than any wait of the ROM kernels can
  if (polls > (1ull << 24))
    return shaw::fail(SHAW_ERR_INVALID_ARG, "polls must be at most 16777216 (the kernels' wait limit)");
  unsigned int s = 0;
  if (int rc = shaw::oz::wait_selftest(polls, &s)) return rc;
  *status = s;
  return SHAW_OK;
}

int shaw_rom_batch_set_tiling(shaw_rom_batch_t h, uint32_t width, int paired) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (!h->oz) return shaw::fail(SHAW_ERR_UNSUPPORTED, "FP64 batches have no tiling");
  return shaw::oz::set_tiling(h->oz, width, paired != 0);
}

int shaw_rom_batch_advance(shaw_rom_batch_t h, double dt, uint64_t nsteps) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (!(dt > 0.0) || !std::isfinite(dt)) return shaw::fail(SHAW_ERR_INVALID_ARG, "dt must be > 0");
  for (const BInst& in : h->inst) {
    if (in.fvp && h->step + nsteps > in.snap_nsteps)
      return shaw::fail(SHAW_ERR_INVALID_ARG, "advancing past the step count the snapshots were sized for");
    if (in.fseis && h->step + nsteps > in.seis_nsteps)
      return shaw::fail(SHAW_ERR_INVALID_ARG, "advancing past the step count the seismogram was sized for");
  }
  if (nsteps == 0) return SHAW_OK;
  if (h->oz) {
    if (int rc = shaw::oz::advance(h->oz, h->stream, dt, h->step, nsteps)) return rc;
    h->launches++;
    h->step += nsteps;
    return SHAW_OK;
  }
  for (uint64_t s = 0; s < nsteps; ++s) {
    if (int rc = fp64_step(h, dt, h->step + 1)) return rc;
    h->step++;
  }
  return SHAW_OK;
}

int shaw_rom_batch_synchronize(shaw_rom_batch_t h) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (h->oz)
    if (int rc = shaw::oz::check(h->oz, h->stream)) return rc;
  for (BInst& in : h->inst) {
    if (!in.fvp) continue;
    SHAW_CUDA(cudaMemcpyAsync(in.host_vp, in.snap_vp, in.kv * (in.snap_nsteps / in.fvp) * in.M * sizeof(double),
                              cudaMemcpyDeviceToHost, h->stream));
    SHAW_CUDA(cudaMemcpyAsync(in.host_sp, in.snap_sp, in.ks * (in.snap_nsteps / in.fsp) * in.M * sizeof(double),
                              cudaMemcpyDeviceToHost, h->stream));
  }
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  return SHAW_OK;
}

int shaw_rom_batch_run(shaw_rom_batch_t h, double dt, uint64_t nsteps) {
  if (int rc = shaw_rom_batch_reset(h)) return rc;
  if (int rc = shaw_rom_batch_advance(h, dt, nsteps)) return rc;
  return shaw_rom_batch_synchronize(h);
}

int shaw_rom_batch_get_state(shaw_rom_batch_t h, uint32_t i, double* xv, double* xs) {
  if (!h || !xv || !xs) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (i >= h->inst.size()) return shaw::fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  const BInst& in = h->inst[i];
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (h->oz) {
    double *dv = nullptr, *ds = nullptr;
    SHAW_CUDA(cudaMalloc(&dv, in.kv * in.M * sizeof(double)));
    if (cudaMalloc(&ds, in.ks * in.M * sizeof(double)) != cudaSuccess) {
      cudaFree(dv);
      return shaw::fail(SHAW_ERR_CUDA, "cudaMalloc (state copy)");
    }
    int rc = shaw::oz::get_state(h->oz, i, h->stream, dv, ds);
    if (rc == SHAW_OK && (cudaMemcpyAsync(xv, dv, in.kv * in.M * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
                          cudaMemcpyAsync(xs, ds, in.ks * in.M * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
                          cudaStreamSynchronize(h->stream) != cudaSuccess))
      rc = shaw::fail(SHAW_ERR_CUDA, "state copy failed");
    cudaFree(dv);
    cudaFree(ds);
    return rc;
  }
  SHAW_CUDA(cudaMemcpyAsync(xv, in.xv, in.kv * in.M * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SHAW_CUDA(cudaMemcpyAsync(xs, in.xs, in.ks * in.M * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  return SHAW_OK;
}

int shaw_rom_batch_describe(shaw_rom_batch_t h, char* out, size_t cap) {
  if (!h || !out || !cap) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  const std::string d = h->oz ? "Ozaki BF16 tensor cores, one persistent launch: " + shaw::oz::describe(h->oz)
                              : "FP64 cuBLAS DGEMM per instance + one batched forcing kernel per step";
  std::strncpy(out, d.c_str(), cap - 1);
  out[cap - 1] = '\0';
  return SHAW_OK;
}

void* shaw_rom_batch_stream(shaw_rom_batch_t h) { return h ? (void*)h->stream : nullptr; }
uint64_t shaw_rom_batch_kernel_launches(shaw_rom_batch_t h) { return h ? h->launches : 0; }
uint64_t shaw_rom_batch_step(shaw_rom_batch_t h) { return h ? h->step : 0; }

}  // extern "C"
