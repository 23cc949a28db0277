// ---------------------------------------------------------------------------
// MapOverlap definitions visible to the user function: the tile geometry,
// input_matrix_t and getData (include/SkelCL/detail/MapOverlapDef.h:205-222).
// getData(m, x, y) reads the staged window at column offset x, row offset y.
// ---------------------------------------------------------------------------
#define SCL_R SCL_OVERLAP_RANGE
#define SCL_TW (32 * SCL_PX)  // tile columns: SCL_PX adjacent columns per thread
// TMA x coordinates must be multiples of 16 bytes: the window starts
// SCL_XLEAD >= R elements left of the tile so that x0 - SCL_XLEAD is aligned.
#define SCL_XALIGN (16 / (int)sizeof(SCL_TYPE_0) > 0 ? 16 / (int)sizeof(SCL_TYPE_0) : 1)
#define SCL_XLEAD (((SCL_R + SCL_XALIGN - 1) / SCL_XALIGN) * SCL_XALIGN)
#define SCL_WIN_W_RAW (SCL_XLEAD + SCL_TW + SCL_R)
#define SCL_WIN_W (((SCL_WIN_W_RAW + SCL_XALIGN - 1) / SCL_XALIGN) * SCL_XALIGN)

typedef struct {
  const SCL_TYPE_0* data;  // the thread's centre element in the staged window
  int local_row;
  int local_column;
} input_matrix_t;
__device__ __forceinline__ SCL_TYPE_1 getData(input_matrix_t m, int x, int y) {
  return (SCL_TYPE_1)m.data[y * SCL_WIN_W + x];
}
