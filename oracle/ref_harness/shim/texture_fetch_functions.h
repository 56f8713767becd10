// Empty stand-in: this header no longer ships with CUDA 13 and the reference kernels use nothing from it.
#pragma once
