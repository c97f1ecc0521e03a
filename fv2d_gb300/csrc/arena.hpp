// arena.hpp -- the chunked first-fit allocator that holds the service's
// simulation states in HBM.
//
// Memory is reserved from the backend in chunks of at least 1 GiB (or just
// the request, when the budget has no room for a full chunk), never more than
// `budget` bytes in total.  Blocks are 256-byte aligned, carved first-fit from
// the chunks' free lists and merged with their free neighbours on release, so
// admitting and retiring simulations does not reserve memory again once the
// arena has grown to the working set.  Chunks are returned only by free_all.
//
// Backend: static void *reserve(size_t bytes) (nullptr on failure) and static
// void unreserve(void *).  The service uses cudaMalloc / cudaFree; the tests
// drive the same code with malloc / free.
#pragma once

#include <algorithm>
#include <cstddef>
#include <iterator>
#include <map>
#include <vector>

namespace fv2d {

template <class Backend>
struct Arena {
  struct Chunk {
    char *base;
    size_t size;
    std::map<size_t, size_t> free;  // offset -> size of each free block
  };
  std::vector<Chunk> chunks;
  double budget = 0;
  size_t reserved = 0, in_use = 0;
  static constexpr size_t kMinChunk = (size_t)1 << 30;

  static size_t align(size_t n) { return (n + 255) & ~size_t(255); }

  // A block of at least n bytes, or nullptr (budget, backend).  A
  // std::bad_alloc from the bookkeeping leaves the arena unchanged.
  void *alloc(size_t n) {
    n = align(n);
    for (auto &c : chunks)
      for (auto it = c.free.begin(); it != c.free.end(); ++it)
        if (it->second >= n) {
          const size_t off = it->first, sz = it->second;
          if (sz > n) c.free.emplace_hint(std::next(it), off + n, sz - n);
          c.free.erase(it);
          in_use += n;
          return c.base + off;
        }
    size_t want = std::max(n, kMinChunk);
    if ((double)(reserved + want) > budget) want = n;
    if ((double)(reserved + want) > budget) return nullptr;
    chunks.reserve(chunks.size() + 1);
    Chunk c{nullptr, want, {}};
    if (want > n) c.free.emplace(n, want - n);
    c.base = static_cast<char *>(Backend::reserve(want));
    if (!c.base) return nullptr;
    chunks.push_back(std::move(c));  // capacity reserved above: does not throw
    reserved += want;
    in_use += n;
    return chunks.back().base;
  }

  // Returns a block of n bytes (the size it was allocated with) at ptr.
  void release(void *ptr, size_t n) {
    n = align(n);
    char *p = static_cast<char *>(ptr);
    for (auto &c : chunks)
      if (p >= c.base && p < c.base + c.size) {
        const size_t off = p - c.base;
        in_use -= n;
        auto next = c.free.lower_bound(off);
        if (next != c.free.end() && next->first == off + n) {  // merge with the following block
          n += next->second;
          next = c.free.erase(next);
        }
        if (next != c.free.begin()) {  // merge with the preceding block
          auto prev = std::prev(next);
          if (prev->first + prev->second == off) {
            prev->second += n;
            return;
          }
        }
        c.free.emplace_hint(next, off, n);
        return;
      }
  }

  void free_all() {
    for (auto &c : chunks) Backend::unreserve(c.base);
    chunks.clear();
    reserved = in_use = 0;
  }
};

}  // namespace fv2d
