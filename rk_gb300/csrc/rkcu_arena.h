// Offsets of the batch's device arena: first-fit allocation, and coalescing
// with the free neighbours on release -- the bookkeeping behind admission by
// HBM footprint (rkcu_batch_add refuses an instance whose footprint fits in
// no free block).  Host code only; tests/native/arena_check.cpp checks it.
#pragma once

#include <algorithm>
#include <cstddef>
#include <vector>

namespace rkcu {

class ArenaList {
 public:
  struct Block {
    size_t off, size;
  };

  // one free block of `bytes`
  void reset(size_t bytes) { blocks_.assign(1, Block{0, bytes}); }

  // The first free block (lowest offset) that holds `size` bytes gives up its
  // lowest `size` bytes; false if none does.
  bool alloc(size_t size, size_t *off) {
    for (size_t i = 0; i < blocks_.size(); ++i) {
      Block &f = blocks_[i];
      if (f.size >= size) {
        *off = f.off;
        f.off += size;
        f.size -= size;
        if (f.size == 0) blocks_.erase(blocks_.begin() + static_cast<std::ptrdiff_t>(i));
        return true;
      }
    }
    return false;
  }

  // [off, off + size) is free again, merged with the free blocks it touches.
  void release(size_t off, size_t size) {
    auto it = std::lower_bound(blocks_.begin(), blocks_.end(), off,
                               [](const Block &f, size_t o) { return f.off < o; });
    it = blocks_.insert(it, Block{off, size});
    size_t i = static_cast<size_t>(it - blocks_.begin());
    if (i + 1 < blocks_.size() && blocks_[i].off + blocks_[i].size == blocks_[i + 1].off) {
      blocks_[i].size += blocks_[i + 1].size;
      blocks_.erase(blocks_.begin() + static_cast<std::ptrdiff_t>(i + 1));
    }
    if (i > 0 && blocks_[i - 1].off + blocks_[i - 1].size == blocks_[i].off) {
      blocks_[i - 1].size += blocks_[i].size;
      blocks_.erase(blocks_.begin() + static_cast<std::ptrdiff_t>(i));
    }
  }

  size_t free_bytes() const {
    size_t n = 0;
    for (const Block &f : blocks_) n += f.size;
    return n;
  }

  // the free blocks by offset (never two adjacent ones)
  const std::vector<Block> &blocks() const { return blocks_; }

 private:
  std::vector<Block> blocks_;
};

}  // namespace rkcu
