// MapOverlap boundary handling (include/SkelCL/detail/Padding.h:45-52 of the
// reference).  SCL_NEUTRAL / SCL_NEAREST are accepted as alternative spellings.
#ifndef SKELCL_PADDING_H_
#define SKELCL_PADDING_H_

namespace skelcl {
namespace detail {

enum class Padding {
  NEUTRAL,
  NEAREST,
  SCL_NEUTRAL = NEUTRAL,
  SCL_NEAREST = NEAREST
};

}  // namespace detail
}  // namespace skelcl

#endif  // SKELCL_PADDING_H_
