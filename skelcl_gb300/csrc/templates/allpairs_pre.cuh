// ---------------------------------------------------------------------------
// Generic AllPairs definitions visible to the user function
// (include/SkelCL/detail/AllPairsDef.h:297-315): lmatrix_t / rmatrix_t keep
// the reference's fields (data, dimension, row / data, width, column) with
// their reference meaning; the accessors read through hidden fields that
// point either at the row / column in global memory or at its staged copy in
// shared memory.
// ---------------------------------------------------------------------------
typedef struct {
  const SCL_TYPE_0* data;
  unsigned int dimension;
  unsigned int row;
  const SCL_TYPE_0* scl_row;
} lmatrix_t;

typedef struct {
  const SCL_TYPE_1* data;
  unsigned int width;
  unsigned int column;
  const SCL_TYPE_1* scl_col;
  unsigned int scl_stride;
} rmatrix_t;

__device__ __forceinline__ SCL_TYPE_0 getElementFromRow(lmatrix_t* m, const unsigned int i) {
  return m->scl_row[i];
}
__device__ __forceinline__ SCL_TYPE_1 getElementFromColumn(rmatrix_t* m, const unsigned int i) {
  return m->scl_col[(size_t)i * m->scl_stride];
}
