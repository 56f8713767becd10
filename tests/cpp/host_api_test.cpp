// Driver for the reference-shaped C++ host classes, used by the tests.
//   host_api_test roundtrip <in.nlos> <out.nlos>         (no GPU)
//   host_api_test shape <in.nlos> <outdir> <V> <filter> <fourier> <aabb>
//   host_api_test lct <in.nlos> <out.cube>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>

#include <cuda_runtime.h>

#include "fbp_reference_api.hpp"

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::string mode = argv[1];
    try {
        if (mode == "roundtrip") {
            NLosData d;
            if (!d.loadBinaryFile(argv[2])) return 3;
            if (!d.saveBinaryFile(argv[3])) return 4;
            std::printf("dims=%zu values=%zu lasers=%zu sensors=%zu T=%u\n", d._dims.size(), d._data.size(),
                        d._laserGridPositions.size(), d._cameraGridPositions.size(), d._temporalResolution);
            return 0;
        }
        if (mode == "shape") {
            NLosData d(argv[2]);
            TransientParameters p;
            p._outputFolder = std::string(argv[3]) + "/";
            p._voxelResolution = fbpref::uvec3((uint32_t)std::atoi(argv[4]));
            p._postprocessingFilterType = (PostprocessingFilterType)std::atoi(argv[5]);
            p._useFourierFilter = std::atoi(argv[6]) != 0;
            p._reconstructAABB = std::atoi(argv[7]) != 0;
            p._numReconstructionDepths = 20;
            Laser laser(&d);
            laser.reconstructShape(p);
            std::printf("ok %zu\n", laser.lastVolume().size());
            return 0;
        }
        if (mode == "mis") {
            NLosData d(argv[2]);
            TransientParameters p;
            p._voxelResolution = fbpref::uvec3(8);
            ReconstructionInfo info;
            ReconstructionBuffers buf;
            d.toGpu(info, buf, p);
            cudaFree(buf._intensity);
            cudaFree(buf._laserTargets);
            cudaFree(buf._sensorTargets);
            float* vol = nullptr;
            if (cudaMalloc(&vol, 512 * sizeof(float)) != cudaSuccess) return 5;
            Laser laser(&d);
            laser.reconstructAABBConfocalMIS(vol, info);
            std::vector<float> h(512);
            cudaMemcpy(h.data(), vol, h.size() * sizeof(float), cudaMemcpyDeviceToHost);
            cudaFree(vol);
            std::ofstream f(argv[3], std::ios::binary);
            f.write(reinterpret_cast<const char*>(h.data()), h.size() * sizeof(float));
            std::printf("ok\n");
            return 0;
        }
        if (mode == "timage") {
            // A 7 x 5 float slice (stride 3, offset 1) enlarged to 13 x 9, and a
            // 4 x 3 uvec4 slice.
            std::vector<float> f(1 + 3 * 35);
            for (size_t i = 0; i < f.size(); ++i) f[i] = (float)((i * 37) % 101) / 97.0f;
            TransientImage a(7, 5);
            a.save(std::string(argv[2]) + "/float.png", f.data(), fbpref::uvec2(13, 9), 3, 1, false);
            std::vector<fbpref::uvec4> u(12);
            for (size_t i = 0; i < u.size(); ++i) u[i] = {(uint32_t)(i * 40), (uint32_t)(300 - i), (uint32_t)i, 7};
            TransientImage b(4, 3);
            b.save(std::string(argv[2]) + "/uvec4.png", u.data());
            std::printf("ok\n");
            return 0;
        }
        if (mode == "images") {
            NLosData d(argv[2]);
            d.saveImages(std::string(argv[3]) + "/");
            std::printf("ok %zu\n", d._dims[0]);
            return 0;
        }
        if (mode == "lct") {
            NLosData d(argv[2]);
            TransientParameters p;
            p._voxelResolution = fbpref::uvec3(4);
            ReconstructionInfo info;
            ReconstructionBuffers buf;
            d.toGpu(info, buf, p);
            LCT lct(info);
            lct.reconstructAABB(info, buf, p);
            std::ofstream f(argv[3], std::ios::binary);
            f.write(reinterpret_cast<const char*>(lct.volume().data()), lct.volume().size() * sizeof(float));
            std::printf("ok %zu\n", lct.volume().size());
            return 0;
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 2;
}
