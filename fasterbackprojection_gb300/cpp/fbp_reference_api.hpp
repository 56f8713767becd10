// C++ host layer with the reference's reconstruction interface, implemented
// on the libfbp C ABI (include/fbp.h).  Class and member names follow the
// reference so a caller of its reconstruction path can switch by swapping
// headers:
//   NLosData              FasterBackprojection/NLosData.h:8-60
//   TransientParameters   FasterBackprojection/TransientParameters.h:5-44
//   ReconstructionInfo / ReconstructionBuffers   GpuStructs.cuh:8-45
//   Laser                 FasterBackprojection/Laser.cuh:14-48
//   LCT                   FasterBackprojection/LCT.h:5-13 (constructor public here)
//   TransientImage        FasterBackprojection/TransientImage.h:7-18
//   PostprocessingFilters, None, Laplacian, LoG, LoGFFT   PostprocessingFilters.h:5-39
// Errors surface as std::runtime_error, like the reference's
// CudaHelper::checkError (CudaHelper.cpp:66-70).  glm is not a dependency:
// the small vec2/vec3/uvec2/uvec3/uvec4 structs below have the same layout.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "fbp.h"

namespace fbpref {
struct vec2 {
    float x = 0, y = 0;
};
struct vec3 {
    float x = 0, y = 0, z = 0;
};
struct uvec3 {
    uint32_t x = 0, y = 0, z = 0;
    uvec3() = default;
    uvec3(uint32_t s) : x(s), y(s), z(s) {}
    uvec3(uint32_t a, uint32_t b, uint32_t c) : x(a), y(b), z(c) {}
};
struct uvec2 {
    uint32_t x = 0, y = 0;
    uvec2() = default;
    explicit uvec2(uint32_t s) : x(s), y(s) {}
    uvec2(uint32_t a, uint32_t b) : x(a), y(b) {}
};
struct uvec4 {
    uint32_t x = 0, y = 0, z = 0, w = 0;
};
}  // namespace fbpref

// GpuStructs.cuh:3-6
enum CaptureSystem : uint32_t { Confocal = 0, Exhaustive = 1 };

// GpuStructs.cuh:8-38: the same 148-byte layout as fbp_recon_info.
using ReconstructionInfo = fbp_recon_info;

// GpuStructs.cuh:40-45: device buffers filled by NLosData::toGpu and freed by
// Laser::reconstructShape (Laser.cu:64-66).
struct ReconstructionBuffers {
    fbpref::vec3* _laserTargets = nullptr;
    fbpref::vec3* _sensorTargets = nullptr;
    float* _intensity = nullptr;
};

// TransientParameters.h:5-11
enum PostprocessingFilterType { NONE, LAPLACIAN, LOG, LOG_FFT, NUM_POSTPROCESSING_FILTERS };

// TransientParameters.h:14-44, same defaults.
class TransientParameters {
public:
    bool _useFourierFilter = true;
    bool _reconstructAABB = true;
    uint32_t _numReconstructionDepths = 200;
    fbpref::uvec3 _voxelResolution{256};
    PostprocessingFilterType _postprocessingFilterType = PostprocessingFilterType::NONE;
    int _kernelSize = 5;
    float _sigma = 1.0f;
    std::string _outputFolder = "output/";
    bool _saveReconstructedBoundingBox = false;
};

// Axis-aligned box (AABB.h:3-25): min/max corners.
struct AABBBox {
    fbpref::vec3 _min{}, _max{};
    fbpref::vec3 minPoint() const { return _min; }
    fbpref::vec3 maxPoint() const { return _max; }
    fbpref::vec3 size() const { return {_max.x - _min.x, _max.y - _min.y, _max.z - _min.z}; }
};

// NLosData.h:8-60.  Loads the reference's ".nlos" binary cache
// (NLosData.cpp:320-405, MSVC x64 layout) or takes arrays directly.
class NLosData {
public:
    std::vector<float> _data;
    std::vector<size_t> _dims;
    std::vector<fbpref::vec3> _cameraGridPositions;
    std::vector<fbpref::vec3> _cameraGridNormals;
    fbpref::vec3 _cameraPosition{};
    fbpref::vec2 _cameraGridSize{};
    std::vector<fbpref::vec3> _laserGridPositions;
    std::vector<fbpref::vec3> _laserGridNormals;
    fbpref::vec3 _laserPosition{};
    fbpref::vec2 _laserGridSize{};
    AABBBox _hiddenGeometry{};
    uint32_t _temporalResolution = 0;
    float _deltaT = 0.f, _t0 = 0.f;
    bool _isConfocal = true;

    NLosData() = default;
    // NLosData.cpp:15-127: filename's ".nlos" twin is read when present (useBinary);
    // this library has no HDF5/MAT reader: other files throw.
    explicit NLosData(const std::string& filename, bool saveBinary = true, bool useBinary = true);
    virtual ~NLosData() = default;

    // NLosData.cpp:131-159: device buffers + geometry.  voxel size = AABB size / resolution.
    void toGpu(ReconstructionInfo& recInfo, ReconstructionBuffers& recBuffers,
               const TransientParameters& transientParameters);

    bool loadBinaryFile(const std::string& filename);
    bool saveBinaryFile(const std::string& filename) const;
    // NLosData.cpp:161-180: "<outPath>transient_<row>.png" per scan row, the
    // [cols][T] slice normalised by its maximum; the directory is created
    // when missing.  Unlike the reference, _data itself is left unchanged
    // (its normalizeImage divides the host slice in place).
    void saveImages(const std::string& outPath);
};

// TransientImage.h:7-18: an RGBA8 image of width x height; save() writes it
// as a PNG file.
class TransientImage {
public:
    TransientImage(uint16_t width, uint16_t height);
    virtual ~TransientImage() = default;
    // TransientImage.cpp:31-44: channels x, y, z clamped to 255, alpha 255,
    // rows flipped.  slice: width * height host values.
    void save(const std::string& filename, const fbpref::uvec4* slice);
    // TransientImage.cpp:46-64: grey pixels clamp(uint(v * 255), 0, 255) of
    // slice[offset + idx * stride] (host memory), rows flipped, bilinearly
    // resized to `size` when it differs (made on the GPU by
    // fbp_transient_images).  normalize divides by the plane's maximum first;
    // unlike the reference, `slice` itself is not modified.
    void save(const std::string& filename, float* slice, const fbpref::uvec2& size, uint32_t stride, uint32_t offset,
              bool normalize = false);
    uint16_t getWidth() const { return _width; }
    uint16_t getHeight() const { return _height; }

private:
    uint16_t _width, _height;
};

// PostprocessingFilters.h:5-39.  compute() replaces `input` with a new device
// buffer holding the filtered volume and frees the old one (the reference's
// pointer swap, PostprocessingFilters.cu:29-31).
class PostprocessingFilters {
public:
    virtual ~PostprocessingFilters() = default;
    virtual void compute(float*& input, const fbpref::uvec3& size, const TransientParameters& p) const = 0;
};
class None : public PostprocessingFilters {
public:
    void compute(float*&, const fbpref::uvec3&, const TransientParameters&) const override {}
};
class Laplacian : public PostprocessingFilters {
public:
    void compute(float*& input, const fbpref::uvec3& size, const TransientParameters& p) const override;
};
class LoG : public PostprocessingFilters {
public:
    static std::vector<float> calculateLaplacianKernel(int size, float std1);
    void compute(float*& input, const fbpref::uvec3& size, const TransientParameters& p) const override;
};
class LoGFFT : public PostprocessingFilters {
public:
    void compute(float*& input, const fbpref::uvec3& size, const TransientParameters& p) const override;
};

// Laser.cuh:14-48
class Laser {
public:
    explicit Laser(NLosData* nlosData);
    virtual ~Laser() = default;

    // Laser.cu:40-67: filter_H, upload, AABB or depth-plane reconstruction,
    // post-filter, normalisation, "<outputFolder>aabb.cube" (AABB mode) or
    // "<outputFolder>depths.raw" (depth mode: float32 [L][D]) plus the depth
    // planes as "<outputFolder>transient_<d>.png" (Laser.cu:409-424, 461-476).
    void reconstructShape(const TransientParameters& transientParams);
    // Laser.cu:526-611: the reference's one-sample MIS (L/4 samples per voxel,
    // default noise buffer; samples summed in order, FBP_MIS_REFERENCE of
    // fbp_mis_backproject) on this capture; `volume` is a device buffer of
    // Vx*Vy*Vz floats.
    void reconstructAABBConfocalMIS(float* volume, const ReconstructionInfo& recInfo) const;

    // The last reconstruction (host copy).
    const std::vector<float>& lastVolume() const { return _lastVolume; }
    // Laser.cu:69-78
    static std::vector<double> linearSpace(double minValue, double maxValue, int n);

private:
    NLosData* _nlosData = nullptr;
    std::vector<float> _lastVolume;
    static const PostprocessingFilters* postprocessingFilter(PostprocessingFilterType t);
};

// LCT.h:5-13 (the reference's implementation is an empty stub, LCT.cpp:16-18).
class LCT {
public:
    explicit LCT(ReconstructionInfo recInfo);
    virtual ~LCT() = default;
    // Confocal LCT of recBuffers._intensity (time-innermost, N x N scan points
    // x T bins); the result [T][N][N] is kept in volume().
    void reconstructAABB(const ReconstructionInfo& recInfo, const ReconstructionBuffers& recBuffers,
                         const TransientParameters& transientParameters);
    const std::vector<float>& volume() const { return _volume; }
    float _snr = 0.8f;
    bool _diffuse = true;

private:
    ReconstructionInfo _info;
    std::vector<float> _volume;
};

// The process-wide libfbp context the classes share (the reference's
// CudaContext singleton, CudaContext.cpp:6-58).
fbp_context* fbp_default_context();
