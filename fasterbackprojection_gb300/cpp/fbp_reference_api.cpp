// Implementation of the reference-shaped host classes on the libfbp C ABI.
#include "fbp_reference_api.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sys/stat.h>


// The reference selects its voxel-scattering kernels at compile time
// (ACCUMULATE_VOXEL_SCATTERING, transient_reconstruction.cuh:112-126,
// 235-250); building this file with the same macro selects the matching
// entry points.
#ifdef ACCUMULATE_VOXEL_SCATTERING
static constexpr auto kConfocalGather = fbp_backproject_confocal_scatter;
static constexpr int kMisReferenceProposal = FBP_MIS_REFERENCE_SCATTER;
#else
static constexpr auto kConfocalGather = fbp_backproject_confocal;
static constexpr int kMisReferenceProposal = FBP_MIS_REFERENCE;
#endif

namespace {

void check(fbp_status st, const char* what) {
    if (st != FBP_OK) throw std::runtime_error(std::string(what) + ": " + fbp_last_error());
}

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// An owned device array of n elements (at least one), optionally filled from
// host memory; freed on scope exit unless released.
template <typename T>
class DeviceArray {
public:
    explicit DeviceArray(size_t n) { check_cuda(cudaMalloc(&_p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc"); }
    DeviceArray(const T* host, size_t n) : DeviceArray(n) {
        if (n) check_cuda(cudaMemcpy(_p, host, n * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    ~DeviceArray() { cudaFree(_p); }
    T* get() const { return _p; }
    T* release() {
        T* p = _p;
        _p = nullptr;
        return p;
    }

private:
    T* _p = nullptr;
};

void make_dirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
    }
    if (!path.empty() && path.back() != '/') mkdir(path.c_str(), 0755);
}

// FileUtilities::write (FileUtilities.h:13-27): raw little-endian values, no header.
bool write_raw(const std::string& filename, const std::vector<float>& v) {
    std::ofstream f(filename, std::ios::binary);
    if (!f.is_open()) return false;
    f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(float));
    return static_cast<bool>(f);
}

}  // namespace

fbp_context* fbp_default_context() {
    static std::once_flag once;
    static fbp_context* ctx = nullptr;
    static fbp_status st = FBP_OK;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        st = fbp_create(&ctx, dev);
    });
    check(st, "fbp_create");
    return ctx;
}

// ------------------------------------------------------------------ NLosData

NLosData::NLosData(const std::string& filename, bool saveBinary, bool useBinary) {
    // NLosData.cpp:17-20: prefer the binary cache next to the capture file.
    const std::string binary = filename.substr(0, filename.find_last_of('.')) + ".nlos";
    if (useBinary && loadBinaryFile(binary)) return;
    if (filename.size() >= 5 && filename.substr(filename.size() - 5) == ".nlos" && loadBinaryFile(filename)) return;
    (void)saveBinary;
    throw std::runtime_error("NLosData: HDF5/MAT captures are not readable by this library (no HDF5 reader); provide the .nlos cache: " +
                             binary);
}

// NLosData.cpp:320-405 (read) / 405-475 (write): sequential raw fields in the
// MSVC x64 layout: vec3 12 B, uint 4 B, float 4 B, bool 1 B, AABB 32 B
// (vptr 8 B, then max and min), size_t 8 B, little endian.
bool NLosData::loadBinaryFile(const std::string& filename) {
    std::ifstream f(filename, std::ios::binary);
    if (!f.is_open()) return false;
    auto rd = [&](void* p, size_t n) {
        f.read(reinterpret_cast<char*>(p), (std::streamsize)n);
        if (!f) throw std::runtime_error("NLosData: truncated .nlos file: " + filename);
    };
    auto rd_size = [&](size_t limit) {
        uint64_t v = 0;
        rd(&v, 8);
        if (v > limit) throw std::runtime_error("NLosData: corrupt .nlos header: " + filename);
        return (size_t)v;
    };
    rd(&_cameraPosition, 12);
    rd(&_laserPosition, 12);
    rd(&_temporalResolution, 4);
    rd(&_deltaT, 4);
    rd(&_t0, 4);
    uint8_t conf = 0;
    rd(&conf, 1);
    _isConfocal = conf != 0;
    unsigned char aabb[32];
    rd(aabb, 32);
    std::memcpy(&_hiddenGeometry._max, aabb + 8, 12);
    std::memcpy(&_hiddenGeometry._min, aabb + 20, 12);
    const size_t nd = rd_size(16);
    _dims.resize(nd);
    for (size_t i = 0; i < nd; ++i) {
        uint64_t d;
        rd(&d, 8);
        _dims[i] = (size_t)d;
    }
    const size_t nc = rd_size(size_t(1) << 32);
    _cameraGridPositions.resize(nc);
    _cameraGridNormals.resize(nc);
    rd(_cameraGridPositions.data(), nc * 12);
    rd(_cameraGridNormals.data(), nc * 12);
    rd(&_cameraGridSize, 8);
    const size_t nl = rd_size(size_t(1) << 32);
    _laserGridPositions.resize(nl);
    _laserGridNormals.resize(nl);
    rd(_laserGridPositions.data(), nl * 12);
    rd(_laserGridNormals.data(), nl * 12);
    rd(&_laserGridSize, 8);
    const size_t nv = rd_size(size_t(1) << 40);
    _data.resize(nv);
    rd(_data.data(), nv * 4);
    size_t prod = 1;
    for (size_t d : _dims) prod *= d;
    if (!_dims.empty() && prod != nv) throw std::runtime_error("NLosData: .nlos dims do not match the data size");
    return true;
}

bool NLosData::saveBinaryFile(const std::string& filename) const {
    std::ofstream f(filename, std::ios::binary);
    if (!f.is_open()) return false;
    auto wr = [&](const void* p, size_t n) { f.write(reinterpret_cast<const char*>(p), (std::streamsize)n); };
    auto wr_size = [&](size_t v) {
        uint64_t x = v;
        wr(&x, 8);
    };
    wr(&_cameraPosition, 12);
    wr(&_laserPosition, 12);
    wr(&_temporalResolution, 4);
    wr(&_deltaT, 4);
    wr(&_t0, 4);
    const uint8_t conf = _isConfocal ? 1 : 0;
    wr(&conf, 1);
    unsigned char aabb[32] = {};
    std::memcpy(aabb + 8, &_hiddenGeometry._max, 12);
    std::memcpy(aabb + 20, &_hiddenGeometry._min, 12);
    wr(aabb, 32);
    wr_size(_dims.size());
    for (size_t d : _dims) wr_size(d);
    wr_size(_cameraGridPositions.size());
    wr(_cameraGridPositions.data(), _cameraGridPositions.size() * 12);
    wr(_cameraGridNormals.data(), _cameraGridNormals.size() * 12);
    wr(&_cameraGridSize, 8);
    wr_size(_laserGridPositions.size());
    wr(_laserGridPositions.data(), _laserGridPositions.size() * 12);
    wr(_laserGridNormals.data(), _laserGridNormals.size() * 12);
    wr(&_laserGridSize, 8);
    wr_size(_data.size());
    wr(_data.data(), _data.size() * 4);
    return static_cast<bool>(f);
}

void NLosData::saveImages(const std::string& outPath) {
    if (_dims.size() > 3) throw std::runtime_error("NLosData: Invalid dimensions for saving images.");
    if (_dims.size() < 3 || _dims[0] == 0) throw std::runtime_error("NLosData: no [rows][cols][T] data to save");
    make_dirs(outPath);
    const size_t slice = _data.size() / _dims[0];
    if (slice != _dims[1] * _dims[2]) throw std::runtime_error("NLosData: dims do not match the data size");
    DeviceArray<float> d(_data.data(), _data.size());
    check(fbp_save_transient_images(fbp_default_context(), d.get(), (uint32_t)_dims[1], (uint32_t)_dims[2],
                                    (uint32_t)_dims[0], 1, slice, (uint32_t)_dims[1], (uint32_t)_dims[2], 1,
                                    outPath.c_str(), nullptr),
          "NLosData::saveImages");
}

void NLosData::toGpu(ReconstructionInfo& in, ReconstructionBuffers& buf, const TransientParameters& tp) {
    std::memset(&in, 0, sizeof(in));
    DeviceArray<float> intensity(_data.data(), _data.size());
    DeviceArray<fbpref::vec3> sensors(_cameraGridPositions.data(), _cameraGridPositions.size());
    DeviceArray<fbpref::vec3> lasers(_laserGridPositions.data(), _laserGridPositions.size());
    buf._intensity = intensity.release();
    buf._sensorTargets = sensors.release();
    buf._laserTargets = lasers.release();
    auto set3 = [](float* d, const fbpref::vec3& v) {
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
    };
    set3(in.sensor_position, _cameraPosition);
    in.num_sensor_targets = (uint32_t)_cameraGridPositions.size();
    set3(in.laser_position, _laserPosition);
    in.num_laser_targets = (uint32_t)_laserGridPositions.size();
    in.num_time_bins = _temporalResolution;
    in.time_step = _deltaT;
    in.time_offset = _t0;
    in.capture_system = _isConfocal ? FBP_CONFOCAL : FBP_EXHAUSTIVE;
    in.discard_first_last_bounces = 0;  // NLosData.cpp:147
    if (!_cameraGridNormals.empty()) set3(in.wall_normal, _cameraGridNormals.front());
    in.wall_min[0] = -_cameraGridSize.x / 2.0f;
    in.wall_min[2] = -_cameraGridSize.y / 2.0f;
    in.wall_size[0] = _cameraGridSize.x;
    in.wall_size[2] = _cameraGridSize.y;
    set3(in.hidden_min, _hiddenGeometry.minPoint());
    set3(in.hidden_max, _hiddenGeometry.maxPoint());
    set3(in.hidden_size, _hiddenGeometry.size());
    in.voxel_res[0] = tp._voxelResolution.x;
    in.voxel_res[1] = tp._voxelResolution.y;
    in.voxel_res[2] = tp._voxelResolution.z;
    // NLosData.cpp:157: size / vec3(resolution), component-wise.
    for (int k = 0; k < 3; ++k) in.voxel_size[k] = in.hidden_size[k] / (float)in.voxel_res[k];
}

// ---------------------------------------------------------------- filters

static void run_filter(fbp_filter kind, float*& input, const fbpref::uvec3& size, const TransientParameters& p) {
    fbp_context* ctx = fbp_default_context();
    DeviceArray<float> out((size_t)size.x * size.y * size.z);
    check(fbp_postfilter(ctx, kind, p._kernelSize, p._sigma, input, out.get(), size.x, size.y, size.z, nullptr),
          "PostprocessingFilters::compute");
    check_cuda(cudaDeviceSynchronize(), "PostprocessingFilters::compute");
    cudaFree(input);
    input = out.release();
}

void Laplacian::compute(float*& input, const fbpref::uvec3& size, const TransientParameters& p) const {
    run_filter(FBP_FILTER_LAPLACIAN, input, size, p);
}
void LoG::compute(float*& input, const fbpref::uvec3& size, const TransientParameters& p) const {
    run_filter(FBP_FILTER_LOG, input, size, p);
}
void LoGFFT::compute(float*& input, const fbpref::uvec3& size, const TransientParameters& p) const {
    run_filter(FBP_FILTER_LOG_FFT, input, size, p);
}
std::vector<float> LoG::calculateLaplacianKernel(int size, float std1) {
    std::vector<float> w((size_t)std::max(size, 0) * size * size);
    check(fbp_log_weights(size, std1, w.data()), "LoG::calculateLaplacianKernel");
    return w;
}

// ------------------------------------------------------------------- Laser

Laser::Laser(NLosData* nlosData) : _nlosData(nlosData) {
    if (!nlosData) throw std::runtime_error("Laser: null NLosData");
}

std::vector<double> Laser::linearSpace(double minValue, double maxValue, int n) {
    std::vector<double> v((size_t)std::max(n, 0));
    if (n > 0) check(fbp_linear_space(minValue, maxValue, n, v.data()), "Laser::linearSpace");
    return v;
}

const PostprocessingFilters* Laser::postprocessingFilter(PostprocessingFilterType t) {
    // Laser.cu:25-30
    static const None none;
    static const Laplacian laplacian;
    static const LoG log;
    static const LoGFFT logfft;
    switch (t) {
        case LAPLACIAN: return &laplacian;
        case LOG: return &log;
        case LOG_FFT: return &logfft;
        default: return &none;
    }
}

void Laser::reconstructShape(const TransientParameters& tp) {
    fbp_context* ctx = fbp_default_context();
    ReconstructionInfo in;
    ReconstructionBuffers buf;
    _nlosData->toGpu(in, buf, tp);
    struct Free {
        ReconstructionBuffers* b;
        ~Free() {
            cudaFree(b->_laserTargets);
            cudaFree(b->_sensorTargets);
            cudaFree(b->_intensity);
        }
    } free_guard{&buf};
    const bool exhaustive = !_nlosData->_isConfocal;
    const uint64_t series = (uint64_t)in.num_laser_targets * (exhaustive ? in.num_sensor_targets : 1);
    // Laser.cu:46-47: filter_H with wl_mean = 10 deltaT (on the device copy).
    if (tp._useFourierFilter)
        check(fbp_filter_h(ctx, buf._intensity, series, in.num_time_bins, in.time_step, in.time_step * 10.0f, 0.0f,
                           FBP_BORDER_ZERO, nullptr),
              "filter_H");
    make_dirs(tp._outputFolder);
    if (tp._reconstructAABB) {
        const size_t V = (size_t)in.voxel_res[0] * in.voxel_res[1] * in.voxel_res[2];
        // The filters replace the buffer they are given (PostprocessingFilters::compute(float*&, ...)).
        float* vol = DeviceArray<float>(V).release();
        try {
            check(exhaustive ? fbp_backproject_exhaustive(ctx, &in, buf._intensity, FBP_F32,
                                                          reinterpret_cast<float*>(buf._laserTargets),
                                                          reinterpret_cast<float*>(buf._sensorTargets), vol, nullptr)
                             : kConfocalGather(ctx, &in, buf._intensity, FBP_F32, FBP_LAYOUT_TIME_INNER,
                                               reinterpret_cast<float*>(buf._laserTargets), vol, nullptr),
                  "backprojection");
            postprocessingFilter(tp._postprocessingFilterType)
                ->compute(vol, fbpref::uvec3(in.voxel_res[0], in.voxel_res[1], in.voxel_res[2]), tp);
            check(fbp_normalize_minmax(ctx, vol, V, nullptr), "normalizeMatrix");
            _lastVolume.resize(V);
            check_cuda(cudaMemcpy(_lastVolume.data(), vol, V * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
        } catch (...) {
            cudaFree(vol);
            throw;
        }
        cudaFree(vol);
        check(fbp_check_device_status(ctx, nullptr), "device status");
        // Laser.cu:361 saveReconstructedAABB("output/aabb.cube").
        if (!write_raw(tp._outputFolder + "aabb.cube", _lastVolume))
            throw std::runtime_error("Laser: cannot write " + tp._outputFolder + "aabb.cube");
        return;
    }
    // Laser.cu:365-377: D depths around the focus depth |(min.y + max.y) / 2|.
    const double focus = std::fabs((in.hidden_min[1] + in.hidden_max[1]) * 0.5f);
    std::vector<double> depths = linearSpace(focus - 0.1f, focus + 0.1f, (int)tp._numReconstructionDepths);
    DeviceArray<double> ddep(depths.data(), depths.size());
    // The activation has num_sensor_targets rows (Laser.cu:389, 441); rows
    // past the laser targets stay zero.
    const uint32_t D = (uint32_t)depths.size();
    const size_t rows = std::max(in.num_laser_targets, in.num_sensor_targets);
    const size_t npix = rows * D;
    DeviceArray<float> act(npix);
    if (rows > in.num_laser_targets)
        check_cuda(cudaMemset(act.get(), 0, npix * sizeof(float)), "cudaMemset");
    check(fbp_backproject_depths(ctx, &in, buf._intensity, FBP_F32, FBP_LAYOUT_TIME_INNER,
                                 reinterpret_cast<float*>(buf._laserTargets),
                                 reinterpret_cast<float*>(buf._sensorTargets), ddep.get(), D, act.get(), nullptr),
          "depth reconstruction");
    check(fbp_normalize_minmax(ctx, act.get(), npix, nullptr), "depth reconstruction");
    _lastVolume.resize(npix);
    check_cuda(cudaMemcpy(_lastVolume.data(), act.get(), npix * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
    // Laser.cu:410-424, 462-476: one image per depth of side sqrt(num_sensor_targets),
    // enlarged to 256 (confocal, when smaller) or 4x (exhaustive).
    const uint32_t side = (uint16_t)std::sqrt((float)in.num_sensor_targets);
    const bool confocal = in.capture_system == FBP_CONFOCAL;
    const uint32_t out = confocal ? side * (side < 256u ? 256u / side : 1u) : side * 4u;
    if (side > 0) {
        make_dirs(tp._outputFolder);
        check(fbp_save_transient_images(ctx, act.get(), side, side, D, D, 1, out, out, 0, tp._outputFolder.c_str(),
                                        nullptr),
              "depth reconstruction");
    }
    if (!write_raw(tp._outputFolder + "depths.raw", _lastVolume))
        throw std::runtime_error("Laser: cannot write " + tp._outputFolder + "depths.raw");
}

void Laser::reconstructAABBConfocalMIS(float* volume, const ReconstructionInfo& recInfo) const {
    // Laser.cu:526-611: the reference's one-sample MIS over L/4 samples per
    // voxel with its default noise buffer, on this capture's data (the
    // reference reads the buffers its last toGpu left in __constant__ memory).
    if (!volume) throw std::runtime_error("Laser::reconstructAABBConfocalMIS: null volume");
    if (!_nlosData->_isConfocal) throw std::runtime_error("Laser::reconstructAABBConfocalMIS: confocal captures only");
    DeviceArray<float> cube(_nlosData->_data.data(), _nlosData->_data.size());
    DeviceArray<fbpref::vec3> lx(_nlosData->_laserGridPositions.data(), _nlosData->_laserGridPositions.size());
    fbp_mis_params prm{};
    prm.proposal = kMisReferenceProposal;
    prm.samples = 0;  // L / 4 (Laser.cu:590)
    check(fbp_mis_backproject(fbp_default_context(), &recInfo, cube.get(), FBP_F32, FBP_LAYOUT_TIME_INNER,
                              reinterpret_cast<const float*>(lx.get()), &prm, volume, nullptr),
          "Laser::reconstructAABBConfocalMIS");
    check_cuda(cudaDeviceSynchronize(), "Laser::reconstructAABBConfocalMIS");
}

// ---------------------------------------------------------- TransientImage

TransientImage::TransientImage(uint16_t width, uint16_t height) : _width(width), _height(height) {}

void TransientImage::save(const std::string& filename, const fbpref::uvec4* slice) {
    if (!slice) throw std::runtime_error("TransientImage::save: null slice");
    const size_t w = _width, h = _height;
    std::vector<uint8_t> rgba(w * h * 4);
    for (size_t y = 0; y < h; ++y)  // row y of the file is row h - 1 - y of the slice
        for (size_t x = 0; x < w; ++x) {
            const fbpref::uvec4& p = slice[(h - 1 - y) * w + x];
            uint8_t* o = &rgba[(y * w + x) * 4];
            o[0] = (uint8_t)std::min<uint32_t>(p.x, 255u);
            o[1] = (uint8_t)std::min<uint32_t>(p.y, 255u);
            o[2] = (uint8_t)std::min<uint32_t>(p.z, 255u);
            o[3] = 255;
        }
    check(fbp_write_png(filename.c_str(), rgba.data(), _width, _height), "TransientImage::save");
}

void TransientImage::save(const std::string& filename, float* slice, const fbpref::uvec2& size, uint32_t stride,
                          uint32_t offset, bool normalize) {
    if (!slice) throw std::runtime_error("TransientImage::save: null slice");
    const size_t n = (size_t)_width * _height;
    std::vector<float> plane(n);
    for (size_t i = 0; i < n; ++i) plane[i] = slice[offset + i * (size_t)stride];
    DeviceArray<float> d(plane.data(), n);
    const size_t bytes = (size_t)size.x * size.y * 4;
    DeviceArray<uint8_t> img(bytes);
    check(fbp_transient_images(fbp_default_context(), d.get(), _width, _height, 1, 1, n, size.x, size.y,
                               normalize ? 1 : 0, img.get(), nullptr),
          "TransientImage::save");
    std::vector<uint8_t> host(bytes);
    check_cuda(cudaMemcpy(host.data(), img.get(), bytes, cudaMemcpyDeviceToHost), "D2H");
    check(fbp_write_png(filename.c_str(), host.data(), size.x, size.y), "TransientImage::save");
}

// --------------------------------------------------------------------- LCT

LCT::LCT(ReconstructionInfo recInfo) : _info(recInfo) {}

void LCT::reconstructAABB(const ReconstructionInfo& in, const ReconstructionBuffers& buf, const TransientParameters&) {
    const uint32_t L = in.num_laser_targets, T = in.num_time_bins;
    const uint32_t N = (uint32_t)std::lround(std::sqrt((double)L));
    if (N * N != L) throw std::runtime_error("LCT: the scan grid must be square");
    fbp_lct_params p{};
    p.width = in.wall_size[0] > 0.f ? in.wall_size[0] * 0.5f : 1.0f;
    p.bin_length = in.time_step;
    p.snr = _snr;
    p.diffuse = _diffuse ? 1 : 0;
    p.grid_mode = FBP_LCT_GRID_REFERENCE;
    DeviceArray<float> vol((size_t)T * L);
    check(fbp_lct(fbp_default_context(), buf._intensity, FBP_LAYOUT_TIME_INNER, N, T, &p, vol.get(), nullptr),
          "LCT::reconstructAABB");
    _volume.resize((size_t)T * L);
    check_cuda(cudaMemcpy(_volume.data(), vol.get(), _volume.size() * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
}
