// Test driver for the library's host linear algebra (compiled by
// tests/test_host_la.py together with adc_ottawa_gb300/csrc/hostla.cpp).
//   hostla_driver sbev <in> <out>:  in = int32 n, int32 kd, n*n doubles
//                                    (column-major); out = n eigenvalues
//   hostla_driver syev <in> <out>:  in = int32 n, n*n doubles; out = n values
//   hostla_driver syevv <in> <out>: as syev; out = n values, then the n*n
//                                    eigenvectors (column-major)
//   hostla_driver heap <in> <out>:  in = int32 n, n doubles; out = n int64
//                                    1-based indices in heapsort order
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace adcgpu {
bool host_syev(int n, const double* A, int lda, double* w, double* V);
bool host_sbev_values(int n, int kd, const double* A, int lda, double* w);
void host_heapsort_index(int64_t n, const double* arr, std::vector<int64_t>& indx);
}

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  FILE* f = std::fopen(argv[2], "rb");
  if (!f) return 3;
  int32_t n = 0, kd = 0;
  if (std::fread(&n, 4, 1, f) != 1) return 4;
  const bool band = std::strcmp(argv[1], "sbev") == 0;
  if (band && std::fread(&kd, 4, 1, f) != 1) return 4;
  const bool heap = std::strcmp(argv[1], "heap") == 0;
  const bool vec = std::strcmp(argv[1], "syevv") == 0;
  std::vector<double> a(heap ? (size_t)n : (size_t)n * n);
  if (std::fread(a.data(), 8, a.size(), f) != a.size()) return 5;
  std::fclose(f);
  FILE* o = std::fopen(argv[3], "wb");
  if (!o) return 6;
  if (heap) {
    std::vector<int64_t> idx;
    adcgpu::host_heapsort_index(n, a.data(), idx);
    std::fwrite(idx.data(), 8, idx.size(), o);
  } else {
    std::vector<double> w(n), V(vec ? (size_t)n * n : 0);
    const bool ok = band ? adcgpu::host_sbev_values(n, kd, a.data(), n, w.data())
                         : adcgpu::host_syev(n, a.data(), n, w.data(), vec ? V.data() : nullptr);
    if (!ok) return 7;
    std::fwrite(w.data(), 8, w.size(), o);
    if (vec) std::fwrite(V.data(), 8, V.size(), o);
  }
  std::fclose(o);
  return 0;
}
