// crc64.cpp -- the reference's CRC64 (src/support/crc64.hpp, crc64.cpp): the
// reflected ECMA-182 polynomial 0xC96C5795D7870F42, table driven, starting
// value and final value as the caller passes them (no inversion).  Used for
// the Parquet price-table checksums (src/option/table/parquet/parquet_io.cpp).
#include <cstdint>

#include "mango_gpu.h"

namespace {

struct Crc64Table {
  uint64_t t[256];
  Crc64Table() {
    const uint64_t poly = 0xC96C5795D7870F42ULL;
    for (uint64_t i = 0; i < 256; ++i) {
      uint64_t c = i;
      for (int j = 0; j < 8; ++j) c = (c & 1) ? (c >> 1) ^ poly : (c >> 1);
      t[i] = c;
    }
  }
};

const Crc64Table& table() {
  static const Crc64Table tab;
  return tab;
}

}  // namespace

extern "C" uint64_t mango_gpu_crc64_update(uint64_t crc, const void* data, uint64_t n) {
  const uint64_t* t = table().t;
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (uint64_t i = 0; i < n; ++i) crc = (crc >> 8) ^ t[static_cast<uint8_t>(crc ^ p[i])];
  return crc;
}
