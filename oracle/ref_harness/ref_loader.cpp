// Oracle harness: loads the reference's own CUDA kernels (compiled, unmodified,
// into oracle/_ref/ref_kernels.cubin by oracle/Makefile) and launches them the
// way the reference's host code does.  Test and benchmark infrastructure only:
// it supplies the bit-exact time-bin source for parity tests and the
// "reference CUDA kernels on the same GPU" timings.
//
// The reference drives its kernels through global __constant__ state
// (FasterBackprojection/GpuStructs.cu:4-16) filled with cudaMemcpyToSymbol
// (FasterBackprojection/Laser.cu:52-55, 598-601).  Here the same symbols are
// looked up in the loaded library and written with cudaMemcpy.
//
// Host launch shapes restated from the reference (file:line):
//   confocal voxel   Laser.cu:482-498  block (16,16,1), grid (ceil(VxVy/16), ceil(L/16), Vz)
//   exhaustive voxel Laser.cu:500-516  block (16,16,1); the reference passes
//                    grid (ceil(LS/16), ceil(VxVy/16), Vz) while the kernel
//                    reads blockIdx.x as the voxel and blockIdx.y as the pair
//                    index, so only min(LS, VxVy) of each are covered.  The
//                    harness launches grid (ceil(VxVy/16), ceil(LS/16), Vz),
//                    which covers every (voxel, pair) the kernel body expects.
//   depth confocal   Laser.cu:394-400  block (16,16,1), grid (ceil(L/16), ceil(L/16), D)
//   depth exhaustive Laser.cu:446-452  block (16,2,1),  grid (ceil(LS/16), ceil(L/2), D)
//   MIS              Laser.cu:590-603  block (16,16,1), grid (ceil(VxVy/16), ceil(K/16), Vz)
//   LoG              PostprocessingFilters.cu:20-26      block (8,8,8)
//   Laplacian        PostprocessingFilters.cu:86-91      block (8,8,8)
//   normalise        Laser.cu:333-334                    block 512
#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <string>

namespace {

// Two builds of the reference kernels: [0] as shipped, [1] with
// ACCUMULATE_VOXEL_SCATTERING; g_lib is the selected one.
cudaLibrary_t g_libs[2] = {nullptr, nullptr};
cudaLibrary_t g_lib = nullptr;
std::string g_err;

struct Uvec3 { unsigned x, y, z; };

int fail(const char* what, cudaError_t e) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return 1;
}

int get_kernel(const char* name, cudaKernel_t* k) {
    if (!g_lib) { g_err = "reference library not loaded"; return 1; }
    cudaError_t e = cudaLibraryGetKernel(k, g_lib, name);
    if (e != cudaSuccess) return fail(name, e);
    return 0;
}

int set_symbol(const char* name, const void* src, size_t bytes) {
    if (!g_lib) { g_err = "reference library not loaded"; return 1; }
    void* dptr = nullptr;
    size_t sz = 0;
    cudaError_t e = cudaLibraryGetGlobal(&dptr, &sz, g_lib, name);
    if (e != cudaSuccess) return fail(name, e);
    if (sz != bytes) { g_err = std::string(name) + ": size mismatch"; return 1; }
    e = cudaMemcpy(dptr, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(name, e);
    return 0;
}

int launch(const char* name, dim3 grid, dim3 block, void** args, cudaStream_t s) {
    cudaKernel_t k;
    if (get_kernel(name, &k)) return 1;
    cudaError_t e = cudaLaunchKernel((const void*)k, grid, block, args, 0, s);
    if (e != cudaSuccess) return fail(name, e);
    return 0;
}

unsigned cdiv(unsigned long long a, unsigned b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

extern "C" {

const char* refk_last_error(void) { return g_err.c_str(); }

// Load the cubin built from the reference sources.
int refk_load(const char* cubin_path) {
    if (g_libs[0]) return 0;
    cudaError_t e = cudaLibraryLoadFromFile(&g_libs[0], cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) { g_libs[0] = nullptr; return fail("cudaLibraryLoadFromFile", e); }
    g_lib = g_libs[0];
    return 0;
}

// Load the ACCUMULATE_VOXEL_SCATTERING build as variant 1.
int refk_load_variant(const char* cubin_path) {
    if (g_libs[1]) return 0;
    cudaError_t e = cudaLibraryLoadFromFile(&g_libs[1], cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) { g_libs[1] = nullptr; return fail("cudaLibraryLoadFromFile", e); }
    return 0;
}

// Select the build the next calls use (0: as shipped, 1: voxel scattering).
int refk_select(int which) {
    if (which < 0 || which > 1 || !g_libs[which]) { g_err = "refk_select: build not loaded"; return 1; }
    g_lib = g_libs[which];
    return 0;
}

// info: 148 bytes laid out as the reference's ReconstructionInfo
// (FasterBackprojection/GpuStructs.cuh:8-38).
int refk_set_state(const void* info, size_t info_bytes, const void* laser_targets,
                   const void* sensor_targets, const void* intensity) {
    if (set_symbol("rtRecInfo", info, info_bytes)) return 1;
    if (set_symbol("laserTargets", &laser_targets, sizeof(void*))) return 1;
    if (set_symbol("sensorTargets", &sensor_targets, sizeof(void*))) return 1;
    if (set_symbol("intensityCube", &intensity, sizeof(void*))) return 1;
    return 0;
}

int refk_set_mis_state(const void* noise, const void* spatial_sum, const void* alias, const void* prob) {
    if (set_symbol("noiseBuffer", &noise, sizeof(void*))) return 1;
    if (set_symbol("spatialSum", &spatial_sum, sizeof(void*))) return 1;
    if (set_symbol("aliasTable", &alias, sizeof(void*))) return 1;
    if (set_symbol("probTable", &prob, sizeof(void*))) return 1;
    return 0;
}

// backprojectConfocalVoxel, accumulating atomically into `volume` (the caller zeroes it).
int refk_confocal_voxel(float* volume, unsigned vx, unsigned vy, unsigned vz, unsigned num_laser, void* stream) {
    unsigned slice = vx * vy;
    void* args[] = {&volume, &slice};
    return launch("_Z24backprojectConfocalVoxelPfj", dim3(cdiv(slice, 16), cdiv(num_laser, 16), vz), dim3(16, 16, 1),
                  args, (cudaStream_t)stream);
}

int refk_exhaustive_voxel(float* volume, unsigned vx, unsigned vy, unsigned vz, unsigned num_laser,
                          unsigned num_sensor, void* stream) {
    unsigned slice = vx * vy;
    unsigned long long pairs = (unsigned long long)num_laser * num_sensor;
    void* args[] = {&volume, &slice};
    return launch("_Z26backprojectExhaustiveVoxelPfj", dim3(cdiv(slice, 16), cdiv(pairs, 16), vz), dim3(16, 16, 1),
                  args, (cudaStream_t)stream);
}

int refk_depth_confocal(float* activation, const double* depths, unsigned num_depths, unsigned num_laser, void* stream) {
    void* args[] = {&activation, &depths, &num_depths};
    return launch("_Z19backprojectConfocalPfPKdj", dim3(cdiv(num_laser, 16), cdiv(num_laser, 16), num_depths),
                  dim3(16, 16, 1), args, (cudaStream_t)stream);
}

int refk_depth_exhaustive(float* activation, const double* depths, unsigned num_depths, unsigned num_laser,
                          unsigned num_sensor, void* stream) {
    unsigned long long pairs = (unsigned long long)num_laser * num_sensor;
    void* args[] = {&activation, &depths, &num_depths};
    return launch("_Z21backprojectExhaustivePfPKdj", dim3(cdiv(pairs, 16), cdiv(num_laser, 2), num_depths),
                  dim3(16, 2, 1), args, (cudaStream_t)stream);
}

int refk_confocal_voxel_mis(const float* spatial_sum, float* volume, const float* noise, const unsigned* alias,
                            const float* prob, unsigned vx, unsigned vy, unsigned vz, unsigned num_samples,
                            unsigned noise_size, void* stream) {
    unsigned slice = vx * vy;
    void* args[] = {&spatial_sum, &volume, &noise, &alias, &prob, &slice, &num_samples, &noise_size};
    return launch("_Z27backprojectConfocalVoxelMISPKfPfS0_PKjS0_jjj",
                  dim3(cdiv(slice, 16), cdiv(num_samples, 16), vz), dim3(16, 16, 1), args, (cudaStream_t)stream);
}

int refk_log_filter(const float* in, float* out, unsigned nx, unsigned ny, unsigned nz, const float* weights,
                    int kernel_size, void* stream) {
    Uvec3 res{nx, ny, nz};
    int half = (kernel_size - 1) / 2;
    void* args[] = {&in, &out, &res, &weights, &kernel_size, &half};
    return launch("_Z9LoGFilterPKfPfN3glm5uvec3ES0_ii", dim3(cdiv(nx, 8), cdiv(ny, 8), cdiv(nz, 8)), dim3(8, 8, 8),
                  args, (cudaStream_t)stream);
}

int refk_laplacian_filter(const float* in, float* out, unsigned nx, unsigned ny, unsigned nz, float filter_size,
                          void* stream) {
    Uvec3 res{nx, ny, nz};
    void* args[] = {&in, &out, &res, &filter_size};
    return launch("_Z15laplacianFilterPKfPfN3glm5uvec3Ef", dim3(cdiv(nx, 8), cdiv(ny, 8), cdiv(nz, 8)),
                  dim3(8, 8, 8), args, (cudaStream_t)stream);
}

// normalizeReconstruction with device-resident max/min (the reference obtains
// them with CUB reductions, Laser.cu:328-331).
int refk_normalize(float* v, unsigned n, const float* max_value, const float* min_value, void* stream) {
    void* args[] = {&v, &n, &max_value, &min_value};
    return launch("_Z23normalizeReconstructionPfjPKfS1_", dim3(cdiv(n, 512)), dim3(512), args, (cudaStream_t)stream);
}

}  // extern "C"
