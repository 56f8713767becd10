// Stand-in for the image library the reference links: only the declarations
// its sources use.  The kernel harness needs nothing from it; the image
// harness (ref_image.cpp) defines SOIL_save_image to hand the pixels back.
#pragma once

enum { SOIL_SAVE_TYPE_TGA = 0, SOIL_SAVE_TYPE_BMP = 1, SOIL_SAVE_TYPE_PNG = 2, SOIL_SAVE_TYPE_DDS = 3 };

int SOIL_save_image(const char* filename, int image_type, int width, int height, int channels,
                    const unsigned char* data);
