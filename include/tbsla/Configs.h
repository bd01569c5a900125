/* Configs.h -- build description that TBSLA's driver programs print
 * (src/includes/tbsla/Configs.h.in, written by the reference's CMake
 * configure step).  Here: the drop-in's own build, the compute in the CUDA
 * library built for sm_103a; the host side compiled by the including
 * program's compiler.  TBSLA_COMPILED_WITH_OMP is left undefined: the
 * drop-in's products run on the GPU, not in OpenMP threads. */
#pragma once

#define CMAKE_CXX_FLAGS ""
#define CMAKE_CXX_FLAGS_DEBUG "-g"
#define CMAKE_CXX_FLAGS_RELEASE "-O3"
#define CMAKE_BUILD_TYPE "Release"
#define OpenMP_CXX_FLAGS "-fopenmp"
#define CMAKE_CXX_COMPILER "c++"
#if defined(__clang__)
#define CMAKE_CXX_COMPILER_ID "Clang"
#elif defined(__GNUC__)
#define CMAKE_CXX_COMPILER_ID "GNU"
#else
#define CMAKE_CXX_COMPILER_ID "unknown"
#endif
#ifdef __VERSION__
#define CMAKE_CXX_COMPILER_VERSION __VERSION__
#else
#define CMAKE_CXX_COMPILER_VERSION "unknown"
#endif
