// SKELCL_COMMON_DEFINITION / SKELCL_ADD_DEFINE
// (include/SkelCL/detail/Macros.h:55-61 of the reference): the definition is
// compiled on the host and appended to the source of every skeleton built
// afterwards.
#ifndef SKELCL_MACROS_H_
#define SKELCL_MACROS_H_

#define SKELCL_CONCATENATE_IMPL(s1, s2) s1##s2
#define SKELCL_CONCATENATE(s1, s2) SKELCL_CONCATENATE_IMPL(s1, s2)
#ifdef __COUNTER__
#define SKELCL_ANONYMOUS_VARIABLE SKELCL_CONCATENATE(skelcl_anonymous, __COUNTER__)
#else
#define SKELCL_ANONYMOUS_VARIABLE SKELCL_CONCATENATE(skelcl_anonymous, __LINE__)
#endif

#define SKELCL_COMMON_DEFINITION(definition) \
  definition                                  \
  static skelcl::detail::RegisterCommonDefinition SKELCL_ANONYMOUS_VARIABLE(#definition);

#define SKELCL_ADD_DEFINE(define) \
  static skelcl::detail::RegisterCommonMacroDefinition SKELCL_ANONYMOUS_VARIABLE(#define, define);

#include "../Source.h"

#endif  // SKELCL_MACROS_H_
