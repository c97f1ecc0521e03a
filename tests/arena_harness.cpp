// Randomised check of the service's state arena (fv2d_gb300/csrc/arena.hpp)
// on the host.  The backend hands out address ranges without memory behind
// them (the arena never touches its blocks), so gigabyte-sized chunks cost
// nothing.  After every operation:
//   * live blocks are 256-byte aligned, lie inside one chunk and do not
//     overlap;
//   * in_use is the sum of the live blocks' aligned sizes and reserved the sum
//     of the chunks' sizes, within the budget;
//   * in every chunk the free blocks and the live blocks tile the chunk
//     exactly, and no two free blocks touch (release merged them);
//   * an allocation failed only if no free block was large enough and a new
//     chunk of that size would exceed the budget (or the backend refused).
// At the end every block is released: each chunk is one free block again.
// Usage: arena_harness <seed> <operations>; prints "ok ..." and exits 0.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <vector>

#include "../fv2d_gb300/csrc/arena.hpp"

namespace {

struct FakeMemory {
  static inline uintptr_t next = (uintptr_t)1 << 40;
  static inline bool refuse = false;
  static inline int reservations = 0;
  static void *reserve(size_t n) {
    if (refuse) return nullptr;
    const uintptr_t p = next;
    next += ((n + 4095) & ~(size_t)4095) + ((size_t)1 << 20);  // a gap between chunks
    ++reservations;
    return reinterpret_cast<void *>(p);
  }
  static void unreserve(void *) { --reservations; }
};

using A = fv2d::Arena<FakeMemory>;

int fails = 0;
void check(bool ok, const char *what, long op) {
  if (!ok && fails++ < 10) std::printf("FAIL at op %ld: %s\n", op, what);
}

void check_invariants(const A &a, const std::map<uintptr_t, size_t> &live, long op) {
  size_t used = 0, reserved = 0;
  for (const auto &c : a.chunks) reserved += c.size;
  check(reserved == a.reserved, "reserved == sum of chunk sizes", op);
  check((double)a.reserved <= a.budget, "reserved within the budget", op);
  uintptr_t prev_end = 0;
  for (const auto &b : live) {
    used += A::align(b.second);
    check(b.first % 256 == 0, "block aligned to 256 bytes", op);
    check(b.first >= prev_end, "live blocks do not overlap", op);
    prev_end = b.first + A::align(b.second);
    int inside = 0;
    for (const auto &c : a.chunks)
      if (b.first >= (uintptr_t)c.base && prev_end <= (uintptr_t)c.base + c.size) ++inside;
    check(inside == 1, "block inside exactly one chunk", op);
  }
  check(used == a.in_use, "in_use == sum of live block sizes", op);
  for (const auto &c : a.chunks) {
    // free blocks and live blocks of this chunk, in address order, tile it
    std::map<size_t, std::pair<size_t, bool>> parts;  // offset -> (size, is_free)
    for (const auto &f : c.free) parts[f.first] = {f.second, true};
    const uintptr_t base = (uintptr_t)c.base;
    for (auto it = live.lower_bound(base); it != live.end() && it->first < base + c.size; ++it)
      parts[it->first - base] = {A::align(it->second), false};
    size_t pos = 0;
    bool prev_free = false;
    for (const auto &p : parts) {
      check(p.first == pos, "free and live blocks tile the chunk", op);
      check(!(prev_free && p.second.second), "no two free blocks touch", op);
      check(p.second.first > 0, "no empty free block", op);
      pos = p.first + p.second.first;
      prev_free = p.second.second;
    }
    check(pos == c.size, "tiling ends at the chunk's end", op);
  }
}

// state sizes of the service: two buffers x four planes of (N + 4) rows x
// pitch floats, pitch = N + 4 rounded up to 32
size_t state_bytes(int N) {
  const size_t pitch = (size_t)(N + 4 + 31) / 32 * 32;
  return sizeof(float) * 8 * (size_t)(N + 4) * pitch;
}

}  // namespace

int main(int argc, char **argv) {
  const unsigned seed = argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u;
  const long ops = argc > 2 ? std::atol(argv[2]) : 20000;
  std::mt19937_64 rng(seed);
  A a;
  a.budget = 6.5e9;
  std::map<uintptr_t, size_t> live;
  std::vector<uintptr_t> order;
  long n_alloc = 0, n_null = 0, n_release = 0;
  for (long op = 0; op < ops; ++op) {
    FakeMemory::refuse = (rng() % 50) == 0;  // the backend refuses now and then
    const bool do_alloc = live.empty() || (rng() % 100) < 55;
    if (do_alloc) {
      // grids 64..4096 (multiples of 32), log-uniform like the request stream
      const double u = std::uniform_real_distribution<double>(std::log(64.0), std::log(4096.0))(rng);
      const int N = std::max(64, (int)(std::exp(u) / 32.0 + 0.5) * 32);
      const size_t n = state_bytes(N);
      size_t largest_free = 0;
      for (const auto &c : a.chunks)
        for (const auto &f : c.free) largest_free = std::max(largest_free, f.second);
      void *p = a.alloc(n);
      if (p) {
        ++n_alloc;
        live[(uintptr_t)p] = n;
        order.push_back((uintptr_t)p);
      } else {
        ++n_null;
        check(largest_free < A::align(n), "no free block was large enough", op);
        check(FakeMemory::refuse || (double)(a.reserved + A::align(n)) > a.budget,
              "a new chunk would exceed the budget", op);
      }
    } else {
      const size_t k = rng() % order.size();
      const uintptr_t p = order[k];
      order[k] = order.back();
      order.pop_back();
      a.release(reinterpret_cast<void *>(p), live[p]);
      live.erase(p);
      ++n_release;
    }
    check_invariants(a, live, op);
  }
  for (uintptr_t p : order) a.release(reinterpret_cast<void *>(p), live[p]);
  live.clear();
  check_invariants(a, live, ops);
  check(a.in_use == 0, "nothing in use after releasing everything", ops);
  for (const auto &c : a.chunks)
    check(c.free.size() == 1 && c.free.begin()->first == 0 && c.free.begin()->second == c.size,
          "each chunk is one free block again", ops);
  const size_t nchunks = a.chunks.size();
  a.free_all();
  check(FakeMemory::reservations == 0 && a.chunks.empty() && a.reserved == 0, "free_all returns every chunk", ops);
  if (fails) return 1;
  std::printf("ok seed=%u ops=%ld allocs=%ld refused=%ld releases=%ld chunks=%zu\n", seed, ops, n_alloc, n_null,
              n_release, nchunks);
  return 0;
}
