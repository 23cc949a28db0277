// Compatibility header: detail::Program lives in detail/Skeleton.h.
#ifndef SKELCL_DETAIL_PROGRAM_H_
#define SKELCL_DETAIL_PROGRAM_H_
#include "Skeleton.h"
#endif
