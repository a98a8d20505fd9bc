// Drives the engine through include/acceles_spmv.hpp in the call order of the reference's
// main() (host_spmv_ucsr.cpp:1066-1113) and prints the results for the Python test to check.
#include <cstdio>
#include <random>
#include <vector>

#include "acceles_spmv.hpp"

int main(int argc, char** argv) {
  const uint32_t rows = 30000, cols = 512;
  const unsigned seed = argc > 1 ? (unsigned)atoi(argv[1]) : 1u;
  uint64_t nnz = aes_gen_matrix(AES_GEN_UNIFORM_DEG, rows, cols, 10, 30, seed, nullptr, nullptr, nullptr);
  std::vector<uint64_t> ptr(rows + 1);
  std::vector<uint32_t> col(nnz), x(nnz);
  std::vector<float> val(nnz);
  aes_gen_matrix(AES_GEN_UNIFORM_DEG, rows, cols, 10, 30, seed, ptr.data(), col.data(), val.data());
  for (uint32_t r = 0; r < rows; r++)
    for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) x[e] = r;
  std::mt19937 gen(seed);
  std::uniform_real_distribution<float> u(0.0f, 1.0f);
  std::vector<float> vec(cols);
  for (auto& v : vec) v = u(gen);
  try {
    aes_params p;
    aes_params_default(&p);
    p.bits = 6;
    p.ck = 512;
    p.split = 32;
    p.k_max = 100;
    aes::SpMV q_spmv(x.data(), col.data(), val.data(), rows, cols, nnz, vec.data(), 0, &p);
    long ns = q_spmv(true, 0);
    std::vector<int32_t> res;
    std::vector<uint32_t> idx;
    q_spmv.Q_read_result(res, idx, 0);
    auto top = q_spmv.read_topk();
    std::printf("ns %ld\n", ns);
    std::printf("query");
    for (float v : vec) std::printf(" %.9g", v);
    std::printf("\ncand");
    for (size_t i = 0; i < idx.size(); i++) std::printf(" %u:%d", idx[i], res[i]);
    std::printf("\ntop");
    for (size_t i = 0; i < top.first.size(); i++) std::printf(" %u:%.9g", top.first[i], top.second[i]);
    std::printf("\n");
  } catch (const aes::Error& e) {
    std::printf("error %d %s\n", e.code, e.what());
    return e.code == AES_ERR_NODEV ? 3 : 1;
  }
  return 0;
}
