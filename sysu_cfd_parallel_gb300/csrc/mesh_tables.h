// Host tables derived from a mesh's topology for the cell kernels: the CSR pattern of the cell
// systems and where every cell-face pair lands in it.
#pragma once
#include <memory>
#include <new>
#include <utility>
#include <vector>

namespace cycas {

// allocator that leaves elements created without a value uninitialised, so that a resize costs
// no pass over the memory (the tables below are written entry by entry on several threads)
template <class T>
struct UninitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() noexcept = default;
  template <class U>
  UninitAlloc(const UninitAlloc<U>&) noexcept {}
  template <class U>
  void construct(U*) noexcept {}
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
using IntTable = std::vector<int, UninitAlloc<int>>;

struct MeshTables {
  // CSR pattern of the cell systems: row i holds i and the cells across its interior faces, in
  // ascending order (the reference's MatSetValues rows, navier_velocity.cpp:370-371, in the
  // column order AIJ keeps)
  IntTable rowptr, col;
  IntTable diag;     // [n] position of (i, i)
  // slot-major [6 n] tables, entry j * n + i for face j of cell i (-1 where j >= cell_nface[i]):
  IntTable face_sm;  // the face (Cell[i].face[j], the reference's order)
  IntTable gface;    // the cell's faces in ascending face order (the gradient's sum order)
  IntTable slot;     // position of (i, neighbour across face j) in col; -1 on boundary faces
};

// Builds the tables of n cells with nf faces (cell_face row-major [6 n]; face_cell2 < 0 on
// boundary faces).  Rows are independent once their lengths are known, so cells are processed in
// parallel on up to 16 host threads; the tables do not depend on the thread count.  Throws
// std::runtime_error for the first cell, in cell order, whose face count is outside 1..6, that
// lists a face outside [0, nf), or a face that does not touch it.
MeshTables mesh_tables(int n, int nf, const int* cell_nface, const int* cell_face, const int* face_cell1,
                       const int* face_cell2);

}  // namespace cycas
