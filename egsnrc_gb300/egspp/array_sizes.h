/* Array sizes of the egs++ application in egs_gpu_dose_application.cpp
 * (every egs++ application directory has one: egs++/egs_advanced_application
 * and the Fortran core size the particle stack and media arrays from it).
 * The transport runs on the GPU, so the host stack stays small. */
#ifndef ARRAY_SIZES_
#define ARRAY_SIZES_
#define MXMED 16
#define MXSTACK 1000
#endif
