#ifndef SKELCL_DLL_H_
#define SKELCL_DLL_H_
#define SKELCL_DLL
#endif
