// Galerkin GEP on the device: data layout shared by the host symbolic phase and the CUDA kernels.
//
// The reference integrates every visited basis pair with a 2-D Gauss-Legendre sum
// (galerkin.rs:73-184, integrals.rs:26-92, 292-354). For the affine, axis-aligned Elems of fem_2d
// (element.rs:33-50) every integrand factors into a u-part times a v-part, so each visit is
//     value = C[block][dir_p][dir_q] * Gu[kind_u][interval_u][i_p][i_q] * Gv[kind_v][interval_v][j_p][j_q]
// where G are 1-D quadrature contractions between shape-function families of the outer Elem (sampled
// over the inner Elem's dyadic sub-interval) and of the inner Elem. The kernels evaluate exactly
// that product, in FP64, for each CSR entry.
#pragma once
#include <stdlib.h>
#include <sys/mman.h>

#include <new>
#include <cstdint>
#include <memory>
#include <type_traits>
#include <utility>
#include <vector>

namespace fem2d {

// 1-D contraction families: G[a][b] = sum_m w_m X_a(s x_m + o) Y_b(x_m)
enum GKind { G_NN = 0, G_DD = 1, G_TT = 2, G_ND = 3, G_DN = 4, G_KINDS = 5 };   // D = T' (tangential derivative)

// A visit block: outer Elem P (its specs start at sp_p) integrated against inner Elem Q (specs at sp_q)
// over Q's region. P == Q for the local-local block.
struct alignas(16) GBlock {
  int32_t sp_p, sp_q;   // offsets into the spec array
  int32_t iu, iv;       // interval ids on the u and v axes
  double ca[4];         // curl-curl constants for (dir_p, dir_q) = UU, UV, VU, VV
  double cb[2];         // L2 constants for UU and VV (UV and VU are exactly zero)
};

// Contribution code: block (32 bits) | p local index (16) | q local index (16)
inline uint64_t make_code(uint32_t blk, uint32_t p, uint32_t q) {
  return ((uint64_t)blk << 32) | ((uint64_t)(p & 0xffff) << 16) | (uint64_t)(q & 0xffff);
}

struct DeviceGEP;   // device buffers (assemble.cu)

// std::vector storage whose resize leaves new elements uninitialised (default-initialised): the
// symbolic phase writes every element of its large arrays, and zeroing them first would cost a full
// serial pass over hundreds of MB at 1M DoFs
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind { using other = NoInitAlloc<U>; };
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) { ::new ((void*)p) U; }
  template <class U, class... Args>
  void construct(U* p, Args&&... args) { ::new ((void*)p) U(std::forward<Args>(args)...); }
  // large arrays (hundreds of MB at 1M DoFs) are first touched by the parallel fill passes: ask for
  // transparent huge pages so that first touch costs far fewer page faults
  static constexpr size_t kLarge = size_t(64) << 20;
  T* allocate(size_t n) {
    const size_t bytes = n * sizeof(T);
    if (bytes >= kLarge) {
      void* p = nullptr;
      if (posix_memalign(&p, size_t(2) << 20, bytes) == 0) {
        madvise(p, bytes, MADV_HUGEPAGE);
        return static_cast<T*>(p);
      }
      throw std::bad_alloc();
    }
    return std::allocator<T>::allocate(n);
  }
  void deallocate(T* p, size_t n) {
    if (n * sizeof(T) >= kLarge) free(p);
    else std::allocator<T>::deallocate(p, n);
  }
};
template <class T>
using HostVec = std::vector<T, NoInitAlloc<T>>;

struct HostGEP {
  int64_t n = 0;                       // DoFs
  int64_t nnz_upper = 0, nnz_full = 0;
  int64_t visits = 0;                  // P_visits of the reference
  int basis = 0, nq_u = 0, nq_v = 0;
  int pmax = 0;                        // table stride - 1 (max order over both axes)
  // full symmetric CSR pattern (A and B share it)
  std::vector<int64_t> row_ptr;        // n + 1
  HostVec<int32_t> col;                // nnz_full
  // contributions: per upper-triangle entry u (rows in order, columns ascending within a row) its visit
  // codes codes[vptr[u] .. vptr[u + 1]) in a fixed order; per full entry the upper entry it mirrors
  // (an entry (r, c) and its transpose (c, r) sum the same visits)
  HostVec<int64_t> vptr;               // nnz_upper + 1
  HostVec<int32_t> fsrc;               // nnz_full
  HostVec<uint64_t> codes;             // visits
  // visit blocks, packed specs, intervals
  std::vector<GBlock> blocks;
  std::vector<double> braw;            // per block, 12 doubles of raw pair geometry (integrate_by_parts)
  std::vector<uint32_t> specs;         // i | j << 8 | dir << 16
  std::vector<double> ivl_s, ivl_o;    // interval scale and offset (index 0 = identity)
  std::vector<double> glq_u_x, glq_u_w, glq_v_x, glq_v_w;
};

}  // namespace fem2d
