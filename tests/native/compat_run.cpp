// Exercises the header-compatible C++ entry points (include/drot_qr.hpp,
// include/drot_glr.hpp) the way reference callers use them
// (core/singleexp_qr.cu, core/multiexp_glr.cu): host-buffer wrappers, and the
// device loop with a caller-prepared warm start (core/drot_qr.hpp:321-346).
// Usage: compat_run <n_rows> <n_cols> <n_groups> <input.bin> <out_prefix>
//   input.bin: float32 C (column-major n_rows x n_cols), then p, then q.
// Writes <out_prefix>_{qrw,qrd,glw}.bin (X) and prints one line per call:
//   name n_iter objective
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "drot_glr.hpp"
#include "drot_qr.hpp"

static void save(const char* prefix, const char* name, const float* x, size_t n) {
  char path[1024];
  std::snprintf(path, sizeof(path), "%s_%s.bin", prefix, name);
  FILE* f = std::fopen(path, "wb");
  std::fwrite(x, sizeof(float), n, f);
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 6) return 2;
  const int nr = std::atoi(argv[1]), nc = std::atoi(argv[2]), G = std::atoi(argv[3]);
  const size_t mn = (size_t)nr * nc;
  std::vector<float> c(mn), p(nr), q(nc);
  FILE* f = std::fopen(argv[4], "rb");
  if (!f || std::fread(c.data(), 4, mn, f) != mn || std::fread(p.data(), 4, nr, f) != (size_t)nr ||
      std::fread(q.data(), 4, nc, f) != (size_t)nc)
    return 3;
  std::fclose(f);
  const float rho = 2.0f, r_weight = 1e-2f, eps = 1e-4f;
  const float step = rho / (float)(nr + nc);
  float dur = 0, prep = 0, obj = 0;
  int nit = 0;

  // Host-buffer QR wrapper (core/singleexp_qr.cu:107-109).
  float* x = quadratic_regularizer_drot_wrapper<float>(c.data(), p.data(), q.data(), nr, nc, step,
                                                       r_weight, 20000, eps, &dur, &prep, &nit,
                                                       &obj, true, true);
  if (!x) return 4;
  std::printf("qr_wrapper %d %.9g\n", nit, obj);
  save(argv[5], "qrw", x, mn);
  std::free(x);

  // Device QR loop with the warm start prepared by the caller, as the
  // reference's PyTorch glue does (pytorch/src/qr_drot_cuda_kernel.cu:107-139).
  const int ws = _q_get_work_size_update_x(nr, nc);
  float *dc, *dp, *dq, *dx, *da, *db, *dphi1, *dphi2, *daux, *drs1;
  cudaMalloc(&dc, mn * 4); cudaMalloc(&dp, nr * 4); cudaMalloc(&dq, nc * 4); cudaMalloc(&dx, mn * 4);
  cudaMalloc(&da, nr * 4); cudaMalloc(&db, nc * 4); cudaMalloc(&dphi1, nr * 4);
  cudaMalloc(&dphi2, nc * 4); cudaMalloc(&daux, 5 * 4);
  cudaMalloc(&drs1, (size_t)nr * ((nc + ws - 1) / ws) * 4);
  cudaMemcpy(dc, c.data(), mn * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dp, p.data(), nr * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dq, q.data(), nc * 4, cudaMemcpyHostToDevice);
  const float n = (float)nr, m = (float)nc;
  const float k = 1.0f * step * n * m - 2.0f;
  std::vector<float> v1(nr, (k + 2.0f) / n / (m + n)), v2(nc, (k + 2.0f) / m / (m + n));
  std::vector<float> va(nr, (k + 1.0f) / n), vb(nc, (k + 1.0f) / m);
  float aux[5] = {0, 0, 0, 0, k + 1.0f};
  cudaMemcpy(dphi1, v1.data(), nr * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dphi2, v2.data(), nc * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(da, va.data(), nr * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(db, vb.data(), nc * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(daux, aux, 20, cudaMemcpyHostToDevice);
  cudaMemset(dx, 0, mn * 4);
  const float scale = 1 + step * r_weight * float(nr + nc);
  quadratic_regularizer_drot<float>(dc, dp, dq, nr, nc, step, scale, r_weight, 20000, eps, ws, dx,
                                    da, nullptr, drs1, nullptr, db, nullptr, nullptr, nullptr,
                                    dphi1, dphi2, daux, &nit, &obj);
  if (nit < 0) return 5;
  std::printf("qr_device %d %.9g\n", nit, obj);
  std::vector<float> hx(mn);
  cudaMemcpy(hx.data(), dx, mn * 4, cudaMemcpyDeviceToHost);
  save(argv[5], "qrd", hx.data(), mn);

  // Host-buffer GL wrapper (core/multiexp_glr.cu).
  x = group_lasso_regularizer_drot_wrapper<float>(c.data(), p.data(), q.data(), nr, nc, G, step,
                                                  r_weight, 20000, eps, &dur, &prep, &nit, &obj,
                                                  true, true);
  if (!x) return 6;
  std::printf("gl_wrapper %d %.9g\n", nit, obj);
  save(argv[5], "glw", x, mn);
  std::free(x);
  return 0;
}
