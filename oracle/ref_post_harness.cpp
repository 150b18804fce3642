// Harness around the reference's own post-processing code (src/cimage.cpp CompileImage,
// src/image.cpp PostRendering_SSAO), compiled in place from the reference tree with
// oracle/ref_stubs_post. Test infrastructure only: it pins the oracle's restatement of
// these two steps and produces golden vectors.
#include <cstdlib>
#include <cstring>

#include "cimage.hpp"
#include "image.h"
#include "Render3D.h"
#include "interface.h"

// globals the two files read (defined by the reference's GUI/main sources)
bool noGUI = true;
bool isPostRendering = false;
int NR_THREADS = 1;
sInterface Interface;
sInterface_data Interface_data;
sNoGUIdata noGUIdata;
GtkWidget *darea = nullptr;
bool paletteViewCreated = false;
sMainWindow renderWindow;
double real_clock(void) { return 0.0; }

extern "C" {

// CompileImage (progressive factor 1) of a float RGB image into RGB16.
void ref_compile_image(int w, int h, const float *image_float, double brightness, double contrast, double gamma,
                       int hdr, unsigned short *image16) {
  cImage img(w, h);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      const float *p = image_float + 3 * ((size_t)y * w + x);
      sRGBfloat px;
      px.R = p[0];
      px.G = p[1];
      px.B = p[2];
      img.PutPixelImage(x, y, px);
    }
  sImageAdjustments adj;
  memset(&adj, 0, sizeof(adj));
  adj.brightness = brightness;
  adj.contrast = contrast;
  adj.imageGamma = gamma;
  sImageSwitches sw;
  memset(&sw, 0, sizeof(sw));
  sw.hdrEnabled = hdr != 0;
  img.SetImageParameters(adj, sw);
  img.progressiveFactor = 1;
  img.CompileImage();
  memcpy(image16, img.GetImage16Ptr(), sizeof(unsigned short) * 3 * (size_t)w * h);
}

// PostRendering_SSAO over an RGB16 image with its z-buffer, opacity and colour layers.
void ref_ssao(int w, int h, const float *zbuffer, const unsigned short *opacity, const unsigned char *colour,
              double persp, int quality, int perspective_type, double global_ilum, unsigned short *image16) {
  cImage img(w, h);
  const size_t n = (size_t)w * h;
  memcpy(img.GetZBufferPtr(), zbuffer, sizeof(float) * n);
  memcpy(img.GetOpacityPtr(), opacity, sizeof(unsigned short) * n);
  memcpy(img.GetColorPtr(), colour, 3 * n);
  memcpy(img.GetImage16Ptr(), image16, sizeof(unsigned short) * 3 * n);
  sImageAdjustments adj;
  memset(&adj, 0, sizeof(adj));
  adj.globalIlum = global_ilum;
  sImageSwitches sw;
  memset(&sw, 0, sizeof(sw));
  img.SetImageParameters(adj, sw);
  img.progressiveFactor = 1;
  PostRendering_SSAO(&img, persp, quality, (enumPerspectiveType)perspective_type, true);
  memcpy(image16, img.GetImage16Ptr(), sizeof(unsigned short) * 3 * n);
}

// PostRendering_DOF with the reference's own code, rand() seeded with `seed` first.
void ref_dof(int w, int h, const float *zbuffer, unsigned short *alpha, unsigned short *image16, double deep,
             double neutral, unsigned int seed) {
  cImage img(w, h);
  const size_t n = (size_t)w * h;
  memcpy(img.GetZBufferPtr(), zbuffer, sizeof(float) * n);
  memcpy(img.GetAlphaBufPtr(), alpha, sizeof(unsigned short) * n);
  memcpy(img.GetImage16Ptr(), image16, sizeof(unsigned short) * 3 * n);
  img.progressiveFactor = 1;
  srand(seed);
  PostRendering_DOF(&img, deep, neutral);
  memcpy(image16, img.GetImage16Ptr(), sizeof(unsigned short) * 3 * n);
  memcpy(alpha, img.GetAlphaBufPtr(), sizeof(unsigned short) * n);
}

}  // extern "C"
