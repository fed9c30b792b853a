// The FP64 engine: egs_transport.cu compiled a second time, for Engine<double>
// only and without fused multiply-adds (--fmad=false, set by the build), so
// that its arithmetic rounds like the CPU oracle's (compiled with
// -ffp-contract=off).  Its kernels and device constants live in namespace
// egsgpu::tu64, apart from the FP32 ones in egsgpu::tu32.
#define EGSGPU_PART_F64 1
#define EGSGPU_TU tu64
#include "egs_transport.cu"
