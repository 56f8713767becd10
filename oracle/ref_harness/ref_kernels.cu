// Oracle harness translation unit: compiles the reference's own CUDA kernel
// headers, unmodified, from the reference tree for sm_103a with the reference's
// code-generation flags (fast math, FMA contraction on).  The graphics/GUI
// headers the reference's precompiled header pulls in are empty stand-ins
// (shim/), and the vector-math types come from the project-written subset in
// shim/glm/glm.hpp.
//
// The output (a cubin under oracle/_ref/) is loaded by ref_loader.cpp with the
// CUDA driver API.  It is test infrastructure: the bit-exact time-bin source
// and the "reference CUDA kernels on the same GPU" timing, never product code.
//
// Kernels provided (reference file:line):
//   backprojectConfocal          FasterBackprojection/transient_reconstruction.cuh:41-64
//   backprojectExhaustive        FasterBackprojection/transient_reconstruction.cuh:66-91
//   backprojectConfocalVoxel     FasterBackprojection/transient_reconstruction.cuh:93-136
//   backprojectExhaustiveVoxel   FasterBackprojection/transient_reconstruction.cuh:138-166
//   backprojectConfocalVoxelMIS  FasterBackprojection/transient_reconstruction.cuh:194-260
//   normalizeReconstruction      FasterBackprojection/transient_postprocessing.cuh:10-17
//   laplacianFilter              FasterBackprojection/transient_postprocessing.cuh:21-50
//   LoGFilter                    FasterBackprojection/transient_postprocessing.cuh:52-83
//   multiplyHK                   FasterBackprojection/fourier.cuh:17-31
#include "GpuStructs.cu"
#include "transient_reconstruction.cuh"
#include "transient_postprocessing.cuh"
#include "fourier.cuh"
