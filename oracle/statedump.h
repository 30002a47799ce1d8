// Tiny tagged binary state-dump writer shared by the reference driver
// (oracle/ref_driver.cpp) and the CPU restatement (oracle/lbdem_oracle.cpp).
//
// TEST INFRASTRUCTURE ONLY: this file belongs to the oracle, which is used
// by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as a
// checker. The CUDA product path never includes it.
//
// Layout (little endian):
//   8-byte magic "LBDMP1\0\0"
//   repeated records:
//     u32 name_len, name bytes, u8 dtype ('d' f64, 'i' i32, 'b' u8, 'q' i64),
//     u32 ndim, u64 shape[ndim], raw data
//   terminated by u32 name_len == 0.
// tests/dumpio.py reads it into a dict of numpy arrays.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace lbdump {

class Writer {
 public:
  explicit Writer(const std::string& path) {
    f_ = std::fopen(path.c_str(), "wb");
    if (f_) std::fwrite("LBDMP1\0\0", 1, 8, f_);
  }
  ~Writer() { close(); }
  bool ok() const { return f_ != nullptr; }
  void close() {
    if (!f_) return;
    uint32_t z = 0;
    std::fwrite(&z, 4, 1, f_);
    std::fclose(f_);
    f_ = nullptr;
  }
  void put(const char* name, char dtype, const void* data, size_t elem,
           std::vector<uint64_t> shape) {
    if (!f_) return;
    uint32_t nl = (uint32_t)std::strlen(name);
    std::fwrite(&nl, 4, 1, f_);
    std::fwrite(name, 1, nl, f_);
    std::fwrite(&dtype, 1, 1, f_);
    uint32_t nd = (uint32_t)shape.size();
    std::fwrite(&nd, 4, 1, f_);
    size_t count = 1;
    for (uint64_t s : shape) {
      std::fwrite(&s, 8, 1, f_);
      count *= (size_t)s;
    }
    if (count) std::fwrite(data, elem, count, f_);
  }
  void d(const char* name, const std::vector<double>& v,
         std::vector<uint64_t> shape = {}) {
    if (shape.empty()) shape = {v.size()};
    put(name, 'd', v.data(), 8, shape);
  }
  void i(const char* name, const std::vector<int32_t>& v,
         std::vector<uint64_t> shape = {}) {
    if (shape.empty()) shape = {v.size()};
    put(name, 'i', v.data(), 4, shape);
  }
  void b(const char* name, const std::vector<uint8_t>& v) {
    put(name, 'b', v.data(), 1, {v.size()});
  }
  void scalar(const char* name, double x) { put(name, 'd', &x, 8, {1}); }
  void scalari(const char* name, int64_t x) { put(name, 'q', &x, 8, {1}); }

 private:
  std::FILE* f_ = nullptr;
};

}  // namespace lbdump
