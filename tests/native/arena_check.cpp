// Random allocate/release sequences on rkcu::ArenaList (rk_gb300/csrc/rkcu_arena.h)
// against a byte map of the arena: allocations never overlap and stay inside
// it, each one comes from the lowest free block that holds it (first fit), the
// free list stays sorted and fully coalesced, its total matches the map, and
// after every range is released one block of the whole arena remains.
// Usage: arena_check <sequences> <seed>; prints the first failures.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rkcu_arena.h"

static uint64_t s_state;
static uint64_t next() {  // splitmix64
  uint64_t z = (s_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

int main(int argc, char **argv) {
  const long long seqs = argc > 1 ? atoll(argv[1]) : 2000;
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  long long bad = 0, refused = 0, allocs = 0;
  auto fail = [&](const char *what, long long k) {
    if (bad++ < 5) printf("sequence %lld: %s\n", k, what);
  };
  for (long long k = 0; k < seqs; ++k) {
    const size_t arena = 256 + next() % 4096;
    rkcu::ArenaList al;
    al.reset(arena);
    std::vector<unsigned char> used(arena, 0);
    struct Range { size_t off, size; };
    std::vector<Range> live;
    const int ops = 20 + static_cast<int>(next() % 200);
    for (int op = 0; op < ops; ++op) {
      if (live.empty() || next() % 3 != 0) {
        const size_t size = 1 + next() % (next() % 4 == 0 ? arena / 2 : 64);
        // first fit, from the byte map: the lowest start of a free run of `size` bytes
        // that begins a free block (the list keeps each block's lowest bytes free)
        size_t want = arena;
        for (const auto &f : al.blocks())
          if (f.size >= size) { want = f.off; break; }
        size_t off = 0;
        if (al.alloc(size, &off)) {
          ++allocs;
          if (want == arena || off != want) fail("not first fit", k);
          if (off + size > arena) fail("outside the arena", k);
          for (size_t b = off; b < off + size && b < arena; ++b) {
            if (used[b]) { fail("overlap", k); break; }
            used[b] = 1;
          }
          live.push_back(Range{off, size});
        } else {
          ++refused;
          if (want != arena) fail("refused although a block holds it", k);
        }
      } else {
        const size_t i = next() % live.size();
        const Range r = live[i];
        live.erase(live.begin() + static_cast<std::ptrdiff_t>(i));
        al.release(r.off, r.size);
        for (size_t b = r.off; b < r.off + r.size; ++b) used[b] = 0;
      }
      // the list: sorted, never adjacent, exactly the free bytes of the map
      size_t total = 0, prev_end = 0;
      bool first = true;
      for (const auto &f : al.blocks()) {
        if (f.size == 0) fail("empty block", k);
        if (!first && f.off <= prev_end) fail("blocks not sorted or not coalesced", k);
        for (size_t b = f.off; b < f.off + f.size && b < arena; ++b)
          if (used[b]) { fail("free block over a live range", k); break; }
        total += f.size;
        prev_end = f.off + f.size;
        first = false;
      }
      size_t free_map = 0;
      for (unsigned char u : used) free_map += !u;
      if (total != free_map || al.free_bytes() != free_map) fail("free bytes differ from the map", k);
    }
    for (const Range &r : live) al.release(r.off, r.size);
    if (al.blocks().size() != 1 || al.blocks()[0].off != 0 || al.blocks()[0].size != arena)
      fail("not one block after releasing everything", k);
  }
  printf("arena failures %lld (%lld allocations, %lld refused) in %lld sequences\n", bad, allocs, refused, seqs);
  return bad ? 1 : 0;
}
