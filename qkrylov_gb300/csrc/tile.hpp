// Tiled SpMV variant (spmv_tile.cu): one CTA applies H to the rows of G outer
// blocks of one inner class, with the blocks' slices of x staged in shared
// memory by asynchronous bulk copies, so the inner-term gathers read shared
// memory and each inner-table entry serves G rows.
#pragma once

#include "fast_common.cuh"

namespace qkg {
namespace tilek {

constexpr int kTileThreads = 256;
constexpr int kMaxG = 4;

// G (<= kMaxG) outer blocks with the same inner class: nblk of a[] are used;
// every block has `width` rows whose inner configurations start at
// inner_state[inner_base]; grp is the inner table's group of the class's
// first row.
struct TileItem {
    uint32_t a[kMaxG];
    uint32_t nblk, width, inner_base, grp;
};
static_assert(sizeof(TileItem) == 32, "tile items are 32 bytes");

// Elements of one block slot in shared memory for blocks of at most max_rows
// rows: the slice starts at the 16-byte boundary at or below the block's
// first row, so a slot holds one 16-byte unit more than the block.
inline uint32_t tile_slot(size_t max_rows, size_t elem_bytes) {
    const size_t per16 = 16 / elem_bytes;  // elements per 16 bytes (2 FP32 complex, 1 FP64 complex)
    return (uint32_t)((max_rows + per16 - 1 + per16 - 1) / per16 * per16);
}
// Dynamic shared memory of one CTA.
inline size_t tile_smem(int G, size_t elem_bytes, uint32_t slot, int n_inner, bool unif, size_t amp_bytes) {
    return (size_t)G * slot * elem_bytes + (unif ? 0 : (size_t)G * 2 * n_inner * amp_bytes);
}
// Largest dynamic shared memory a tile CTA may ask for.
constexpr size_t kTileSmemLimit = 220 * 1024;

// Class-persistent SpMV (spmv_class_kernel): one 1024-thread CTA per SM walks
// every grid-th block of a list sorted by inner class; the class's inner
// table is copied into shared memory once per class, each block's slice of x
// arrives by bulk copy into one of two buffers while the previous block is
// computed, and a thread holds four columns of the class.
constexpr int kClassThreads = 1024;
constexpr int kClassCols = 4;  // columns per thread: classes up to 4096 configurations
struct CBlock {
    uint32_t a, cls;
};
struct CClass {
    uint32_t W, inner_base, gbase, ngroups, ell0, ell1;
};
struct ClassPlan {
    const CBlock* blocks;
    const CClass* classes;
    uint32_t nblocks;
    uint32_t slot;     // elements of one slice buffer
    uint32_t ell_cap;  // inner-table entries of the largest class
    uint32_t gcap;     // groups of the largest class
};
// Dynamic shared memory: two slices, the table and its group offsets (padded
// to 16 bytes), then the inner amplitudes of the current block (!unif).
inline size_t class_smem(const ClassPlan& c, size_t elem_bytes, int n_inner, bool unif, size_t amp_bytes) {
    return 2 * (size_t)c.slot * elem_bytes + (((size_t)c.ell_cap + c.gcap + 1) * 4 + 15) / 16 * 16 +
           (unif ? 0 : 2 * (size_t)n_inner * amp_bytes);
}
template <class T, class A>
void launch_class(const fastk::FastParams<A>& p, const ClassPlan& plan, unsigned grid, bool real, bool unif,
                  const typename fastk::V2<T>::t* x, typename fastk::V2<T>::t* y, size_t smem, cudaStream_t s);

template <class T, class A>
void launch_tile(const fastk::FastParams<A>& p, const TileItem* items, size_t n_items, int G, bool real, bool unif,
                 const typename fastk::V2<T>::t* x, typename fastk::V2<T>::t* y, uint32_t slot, size_t smem,
                 cudaStream_t s);
// Raise the dynamic shared-memory limit of every tile kernel of this element
// type on the current device to kTileSmemLimit (once per device; bytes > 0 is
// the Hamiltonian's need, 0 does nothing).
template <class T, class A>
void tile_allow_smem(size_t bytes);

// Bulk-copy waits of the tile kernels that gave up on the current GPU.
uint32_t tile_wait_timeouts();

}  // namespace tilek
}  // namespace qkg
