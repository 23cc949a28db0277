// Host mirrors of the OpenCL vector types (include/SkelCL/detail/Types.h:43-152
// of the reference): plain structs with members s0, s1, ... and no padding,
// laid out exactly like the device-side types of the CUDA prelude.
#ifndef SKELCL_TYPES_H_
#define SKELCL_TYPES_H_

namespace skelcl {

#define SKELCL_VECTOR_TYPES(T, N)                                                   \
  typedef struct { T s0, s1; } N##2;                                                \
  typedef struct { T s0, s1, s2, s3; } N##4;                                        \
  typedef N##4 N##3;                                                                \
  typedef struct { T s0, s1, s2, s3, s4, s5, s6, s7; } N##8;                        \
  typedef struct { T s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf; } N##16;

SKELCL_VECTOR_TYPES(char, char)
SKELCL_VECTOR_TYPES(unsigned char, uchar)
SKELCL_VECTOR_TYPES(short, short)
SKELCL_VECTOR_TYPES(unsigned short, ushort)
SKELCL_VECTOR_TYPES(int, int)
SKELCL_VECTOR_TYPES(unsigned int, uint)
SKELCL_VECTOR_TYPES(long, long)
SKELCL_VECTOR_TYPES(unsigned long, ulong)
SKELCL_VECTOR_TYPES(float, float)
SKELCL_VECTOR_TYPES(double, double)

#undef SKELCL_VECTOR_TYPES

}  // namespace skelcl

#endif  // SKELCL_TYPES_H_
