// Host launchers for the reference's own `gpu`-backend kernels (test infrastructure only).
//
// The reference keeps its device code as CUDA C source in a Rust string (KERNEL_SRC,
// crates/riga-engine/src/gpu.rs:27-76) and compiles it with NVRTC at run time using only
// --gpu-architecture (gpu.rs:84-131), i.e. NVRTC's defaults: -fmad=true, IEEE division and square
// root, no fast math.  ref_gpu.py extracts that string verbatim into _ref/gpu_rs_kernels.cu and
// compiles this file with nvcc's identical defaults, so the kernels below compute what the
// reference's `gpu` backend computes.  The launches follow gpu.rs:171-205 and 209-277: one thread
// per element, cudarc's LaunchConfig::for_num_elems (1024-thread blocks), legacy default stream.
// These launchers are the GPU-side oracle of the drop-in tests; the product never links them.
#include <cuda_runtime.h>

#include "_ref/gpu_rs_kernels.cu"

namespace {
int fail(cudaError_t e) { return e == cudaSuccess ? 0 : (int)e; }

template <class T>
cudaError_t upload(T** d, const T* h, size_t n) {
  cudaError_t e = cudaMalloc(d, sizeof(T) * (n ? n : 1));
  if (e == cudaSuccess && n) e = cudaMemcpy(*d, h, sizeof(T) * n, cudaMemcpyHostToDevice);
  return e;
}
}  // namespace

extern "C" int ref_worst_of(const float* a, const float* b, float* out, int n) {
  float *da = nullptr, *db = nullptr, *dout = nullptr;
  cudaError_t e = upload(&da, a, (size_t)n);
  if (e == cudaSuccess) e = upload(&db, b, (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(float) * (n ? n : 1));
  if (e == cudaSuccess && n > 0) {
    worst_of<<<(unsigned)((n + 1023) / 1024), 1024>>>(da, db, dout, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(out, dout, sizeof(float) * n, cudaMemcpyDeviceToHost);
  cudaFree(da);
  cudaFree(db);
  cudaFree(dout);
  return fail(e);
}

extern "C" int ref_lv_propagate(const float* normals, const float* rows, const float* ls_axis, int gx,
                                const float* s0, float ref0, float ref1, float ko_bar, int paths,
                                int steps, float dt, float rate, float q0, float q1, float* out,
                                int* ko_out) {
  float *dn = nullptr, *dr = nullptr, *dl = nullptr, *ds = nullptr, *dout = nullptr;
  int* dko = nullptr;
  cudaError_t e = upload(&dn, normals, (size_t)paths * steps * 2);
  if (e == cudaSuccess) e = upload(&dr, rows, (size_t)2 * steps * gx);
  if (e == cudaSuccess) e = upload(&dl, ls_axis, (size_t)2 * gx);
  if (e == cudaSuccess) e = upload(&ds, s0, (size_t)2);
  if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(float) * 2 * (paths ? paths : 1));
  if (e == cudaSuccess) e = cudaMalloc(&dko, sizeof(int) * (paths ? paths : 1));
  if (e == cudaSuccess && paths > 0) {
    lv_propagate<<<(unsigned)((paths + 1023) / 1024), 1024>>>(dn, dr, dl, ds, dout, dko, ref0, ref1, ko_bar,
                                                              paths, steps, gx, dt, rate, q0, q1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess && paths > 0) e = cudaMemcpy(out, dout, sizeof(float) * 2 * paths, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && paths > 0) e = cudaMemcpy(ko_out, dko, sizeof(int) * paths, cudaMemcpyDeviceToHost);
  cudaFree(dn);
  cudaFree(dr);
  cudaFree(dl);
  cudaFree(ds);
  cudaFree(dout);
  cudaFree(dko);
  return fail(e);
}
