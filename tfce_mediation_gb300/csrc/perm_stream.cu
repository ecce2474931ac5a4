// Permutation index streams of the mmr-lr convention: row p is
// numpy.random.RandomState(seed + p).permutation(n)
// (tfce_mediation/tm_func.py:147-151, tm_multisurface/tm_mmr_rand_low_ram.py),
// generated natively so that a permutation loop's host side does not spend
// ~0.1 ms of Python per permutation creating a RandomState.
//
// The stream is reproduced exactly from the published algorithms numpy's
// legacy RandomState composes:
//   * MT19937 (Matsumoto & Nishimura 1998), seeded from one 32-bit integer by
//     the reference initialisation key[0] = s, key[i] = 1812433253 *
//     (key[i-1] ^ (key[i-1] >> 30)) + i, and tempered 32-bit outputs;
//   * permutation(n) = shuffle(arange(n)): for i = n-1 down to 1, swap
//     element i with element j drawn uniformly from [0, i] by masked
//     rejection (the smallest all-ones mask >= i, 32-bit draws ANDed with it
//     until one is <= i).
// Host code only (no device work); rows are split over threads.
#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

#include "common.cuh"

namespace tfgb {
namespace {

constexpr int kMtN = 624, kMtM = 397;
constexpr uint32_t kMtMatrixA = 0x9908b0dfu, kMtUpper = 0x80000000u, kMtLower = 0x7fffffffu;

struct Mt19937 {
  uint32_t key[kMtN];
  int pos;

  explicit Mt19937(uint32_t s) {
    key[0] = s;
    for (int i = 1; i < kMtN; ++i) key[i] = 1812433253u * (key[i - 1] ^ (key[i - 1] >> 30)) + static_cast<uint32_t>(i);
    pos = kMtN;
  }

  void twist() {
    for (int i = 0; i < kMtN; ++i) {
      const uint32_t y = (key[i] & kMtUpper) | (key[(i + 1) % kMtN] & kMtLower);
      key[i] = key[(i + kMtM) % kMtN] ^ (y >> 1) ^ ((y & 1u) ? kMtMatrixA : 0u);
    }
    pos = 0;
  }

  uint32_t next() {
    if (pos >= kMtN) twist();
    uint32_t y = key[pos++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }

  // uniform on [0, hi] by masked rejection (hi < 2^32)
  uint32_t interval(uint32_t hi) {
    if (hi == 0) return 0;
    uint32_t mask = hi;
    mask |= mask >> 1;
    mask |= mask >> 2;
    mask |= mask >> 4;
    mask |= mask >> 8;
    mask |= mask >> 16;
    uint32_t v;
    while ((v = next() & mask) > hi) {
    }
    return v;
  }
};

void fill_rows(int64_t n, int64_t seed, int64_t r0, int64_t r1, int64_t* out) {
  for (int64_t r = r0; r < r1; ++r) {
    int64_t* row = out + r * n;
    for (int64_t i = 0; i < n; ++i) row[i] = i;
    Mt19937 mt(static_cast<uint32_t>(seed + r));
    for (int64_t i = n - 1; i >= 1; --i) {
      const int64_t j = mt.interval(static_cast<uint32_t>(i));
      const int64_t t = row[i];
      row[i] = row[j];
      row[j] = t;
    }
  }
}

}  // namespace
}  // namespace tfgb

extern "C" int perm_stream(int64_t n, int64_t seed, int64_t start, int64_t stop, int64_t* out, int32_t threads) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(n >= 0 && n <= 0xffffffffLL, "n must be in [0, 2^32)");
  TFGB_CHECK_ARG(stop >= start, "stop must be >= start");
  if (stop == start) return TFCE_OK;
  TFGB_CHECK_ARG(out != nullptr, "NULL pointer");
  // RandomState accepts seeds in [0, 2^32 - 1] only
  TFGB_CHECK_ARG(seed + start >= 0 && seed + stop - 1 <= 0xffffffffLL, "seed + p must be in [0, 2^32 - 1]");
  const int64_t rows = stop - start;
  const int64_t first = seed + start;
  int64_t nt = threads > 0 ? threads : static_cast<int64_t>(std::thread::hardware_concurrency());
  nt = std::max<int64_t>(1, std::min<int64_t>({nt, 64, (rows * (n + 1000) + 199999) / 200000}));
  if (nt == 1) {
    tfgb::fill_rows(n, first, 0, rows, out);
    return TFCE_OK;
  }
  std::vector<std::thread> pool;
  const int64_t per = (rows + nt - 1) / nt;
  int64_t done = 0;  // rows handed to threads
  for (int64_t t = 0; t < nt; ++t) {
    const int64_t r0 = t * per, r1 = std::min(rows, r0 + per);
    if (r0 >= r1) break;
    try {
      pool.emplace_back(tfgb::fill_rows, n, first, r0, r1, out);
    } catch (...) {
      break;  // no more threads: the calling thread fills the rest
    }
    done = r1;
  }
  if (done < rows) tfgb::fill_rows(n, first, done, rows, out);
  for (auto& th : pool) th.join();
  return TFCE_OK;
}
