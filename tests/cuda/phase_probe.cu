// Device-function probe for tests/test_phase_function.py: evaluates the
// library's exp(z) - 1 and psi * exp(z) helpers (common.cuh) on float
// exponents read from a file and writes the results back.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "common.cuh"

__global__ void probe(const float2 *z, float2 *em1, float2 *mul, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  em1[i] = dftgpu::cexpm1(z[i]);
  mul[i] = dftgpu::mul_cexp(make_float2(0.6f, -0.8f), z[i]);
}

int main(int argc, char **argv) {
  if (argc != 3) { fprintf(stderr, "usage: phase_probe in.bin out.bin\n"); return 2; }
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  std::vector<float2> z;
  float2 v;
  while (fread(&v, sizeof(v), 1, f) == 1) z.push_back(v);
  fclose(f);
  const int n = (int) z.size();
  float2 *dz, *de, *dm;
  if (cudaMalloc(&dz, n * sizeof(float2)) || cudaMalloc(&de, n * sizeof(float2)) || cudaMalloc(&dm, n * sizeof(float2)))
    return 4;
  cudaMemcpy(dz, z.data(), n * sizeof(float2), cudaMemcpyHostToDevice);
  probe<<<(n + 255) / 256, 256>>>(dz, de, dm, n);
  std::vector<float2> e(n), m(n);
  if (cudaMemcpy(e.data(), de, n * sizeof(float2), cudaMemcpyDeviceToHost) ||
      cudaMemcpy(m.data(), dm, n * sizeof(float2), cudaMemcpyDeviceToHost))
    return 5;
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 6;
  fwrite(e.data(), sizeof(float2), n, o);
  fwrite(m.data(), sizeof(float2), n, o);
  fclose(o);
  return 0;
}
