// mbgb_cli: the -nogui entry of Mandelbulber 1.21 on libmbgb.
//
// Command line as ReadComandlineParams (src/interface.cpp:3334-3540):
//   mbgb_cli [options...] [settings_file]        (default settings file: default.fract)
//     -nogui                 accepted (there is no GUI)
//     -flight                flight animation: camera per frame from file_animation_path
//     -keyframe              keyframe animation: file_keyframes00000.fract, 00001, ...
//     -start N / -end N      frame range of the animation
//     -format jpg|png|png16|png16alpha
//     -res WIDTHxHEIGHT      override image_width / image_height
//     -fpk N                 override frames_per_keyframe
//     -o key=value           override one setting
//   options of mbgb_cli only:
//     -defaults FILE         settings read before the settings file (default: none)
//     -precision fp64|fp32|auto    render policy (default fp32: FP32 with FP64 refinement)
//     -batch N               frames rendered per launch sequence (default 16)
//     -device N              CUDA device
// The frame loop follows MainRender (src/Render3D.cpp:1940-2480): frames whose output file
// exists are skipped, keyframe frames come from the Catmull-Rom splines of the keyframes,
// flight frames read "x y z alpha beta gamma" per line; each frame is rendered, compiled
// to 16 bits (CompileImage), post-processed with SSAO when post_SSAO_enabled is set and with
// the depth of field when post_DOF_enabled is set, and
// written as IndexFilename(file_destination, ext, frame) = destination%05d.ext.
// JPEG needs libjpeg, which mbgb_cli does not link: -format jpg writes an 8-bit PNG.
// Network rendering (-ip, -port) and tiled output are not supported by mbgb_cli.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mbgb.h"

namespace {

enum Format { kJPG, kPNG, kPNG16, kPNG16Alpha };

struct Args {
  bool flight = false, keyframe = false;
  int start = 0, end = 99999;
  Format format = kJPG;
  std::vector<std::string> overrides;
  std::string settings = "default.fract";
  std::string defaults;
  int precision = MBGB_PREC_FP32_FIX;
  int batch = 16;
  int device = 0;
};

void usage() {
  printf("Syntax:\nmbgb_cli [options...] [settings_file]\n");
  printf("options:\n");
  printf("  -nogui            - accepted; there is no GUI\n");
  printf("  -flight           - render flight animation\n");
  printf("  -keyframe         - render keyframe animation\n");
  printf("  -start N          - start rendering from frame number N\n");
  printf("  -end N            - rendering will end on frame number N\n");
  printf("  -o key=value      - override item 'key' from settings file with new value 'value'\n");
  printf("  -res WIDTHxHEIGHT - override image resolution\n");
  printf("  -fpk N            - override frames per key parameter\n");
  printf("  -format FORMAT    - image format: jpg (written as 8-bit PNG), png, png16, png16alpha\n");
  printf("  -defaults FILE    - settings file read before the settings file\n");
  printf("  -precision P      - fp64, fp32 (FP32 with FP64 refinement) or auto\n");
  printf("  -batch N          - frames per launch sequence\n");
  printf("  -device N         - CUDA device\n");
}

bool parse(int argc, char **argv, Args &a) {
  for (int i = 1; i < argc; i++) {
    const std::string s = argv[i];
    auto next = [&](const char *what) -> const char * {
      if (i + 1 >= argc) {
        printf("commandline: %s needs an argument\n", what);
        return nullptr;
      }
      return argv[++i];
    };
    if (s == "-nogui") continue;
    if (s == "-flight") { a.flight = true; continue; }
    if (s == "-keyframe") { a.keyframe = true; continue; }
    if (s == "-start" || s == "-end" || s == "-fpk" || s == "-batch" || s == "-device") {
      const char *v = next(s.c_str());
      if (!v) return false;
      const int n = atoi(v);
      if (s == "-start") a.start = n;
      else if (s == "-end") a.end = n;
      else if (s == "-batch") a.batch = n > 0 ? n : 1;
      else if (s == "-device") a.device = n;
      else {
        if (n <= 0) { printf("commandline: argument must be -fpk NNN\n"); return false; }
        a.overrides.push_back("frames_per_keyframe=" + std::to_string(n));
      }
      continue;
    }
    if (s == "-format") {
      const char *v = next("-format");
      if (!v) return false;
      const std::string f = v;
      if (f == "jpg") a.format = kJPG;
      else if (f == "png") a.format = kPNG;
      else if (f == "png16") a.format = kPNG16;
      else if (f == "png16alpha") a.format = kPNG16Alpha;
      else { printf("commandline: wrong image format\n"); return false; }
      continue;
    }
    if (s == "-res") {
      const char *v = next("-res");
      int w, h;
      if (!v || sscanf(v, "%dx%d", &w, &h) != 2) { printf("commandline: Argument must be -res WWWWxHHHH\n"); return false; }
      a.overrides.push_back("image_width=" + std::to_string(w));
      a.overrides.push_back("image_height=" + std::to_string(h));
      continue;
    }
    if (s == "-o") {
      const char *v = next("-o");
      if (!v) return false;
      a.overrides.push_back(v);
      continue;
    }
    if (s == "-defaults") {
      const char *v = next("-defaults");
      if (!v) return false;
      a.defaults = v;
      continue;
    }
    if (s == "-precision") {
      const char *v = next("-precision");
      if (!v) return false;
      const std::string p = v;
      if (p == "fp64") a.precision = MBGB_PREC_FP64;
      else if (p == "fp32") a.precision = MBGB_PREC_FP32_FIX;
      else if (p == "auto") a.precision = MBGB_PREC_AUTO;
      else { printf("commandline: precision must be fp64, fp32 or auto\n"); return false; }
      continue;
    }
    if (s == "-ip" || s == "-port") {
      printf("commandline: network rendering is not supported by mbgb_cli\n");
      return false;
    }
    if (s == "-help" || i < argc - 1) return false;
    a.settings = s;
  }
  return true;
}

std::string index_filename(const std::string &base, const char *ext, int n) {
  char tmp[16];
  snprintf(tmp, sizeof(tmp), "%.5i", n);
  return base + tmp + "." + ext;
}

bool exists(const std::string &path) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return false;
  fclose(f);
  return true;
}

struct Job {
  int index;
  mbgb_scene scene;
  std::string file;
};

#define CLI_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      fprintf(stderr, "mbgb_cli: %s: %s\n", #call, cudaGetErrorString(e_));              \
      return false;                                                                      \
    }                                                                                    \
  } while (0)

// Render a batch of frames, post-process them on the device and write their files.
bool render_jobs(mbgb_context *ctx, const std::vector<Job> &jobs, const Args &a) {
  if (jobs.empty()) return true;
  const size_t n = jobs.size();
  size_t total = 0;
  std::vector<size_t> base(n);
  for (size_t i = 0; i < n; i++) {
    base[i] = total;
    total += (size_t)jobs[i].scene.image_width * jobs[i].scene.image_height;
  }
  // per pixel: float RGB 12, z 4, alpha 2, opacity 2, colour 3, RGB16 6 (29 bytes), padded
  char *dev = nullptr;
  const size_t bytes = total * 32 + n * 6 * 256;
  CLI_CUDA(cudaMalloc(&dev, bytes));
  std::vector<mbgb_image> outs(n);
  std::vector<uint16_t *> img16(n);
  size_t off = 0;
  auto take = [&](size_t b) {
    char *p = dev + off;
    off += (b + 255) & ~(size_t)255;
    return p;
  };
  for (size_t i = 0; i < n; i++) {
    const size_t px = (size_t)jobs[i].scene.image_width * jobs[i].scene.image_height;
    mbgb_image &o = outs[i];
    memset(&o, 0, sizeof(o));
    o.width = jobs[i].scene.image_width;
    o.height = jobs[i].scene.image_height;
    o.image_float = (float *)take(px * 12);
    o.zbuffer = (float *)take(px * 4);
    o.alpha = (uint16_t *)take(px * 2);
    o.opacity = (uint16_t *)take(px * 2);
    o.colour = (uint8_t *)take(px * 3);
    img16[i] = (uint16_t *)take(px * 6);
  }
  std::vector<mbgb_scene> scenes(n);
  for (size_t i = 0; i < n; i++) scenes[i] = jobs[i].scene;
  mbgb_opts opts;
  memset(&opts, 0, sizeof(opts));
  opts.precision = a.precision;
  bool ok = mbgb_render_batch(ctx, scenes.data(), (int32_t)n, outs.data(), &opts) == MBGB_OK;
  if (!ok) fprintf(stderr, "mbgb_cli: render: %s\n", mbgb_last_error());
  std::vector<uint16_t> host16, hostAlpha;
  std::vector<uint8_t> host8;
  for (size_t i = 0; ok && i < n; i++) {
    const mbgb_scene &sc = jobs[i].scene;
    const int w = sc.image_width, h = sc.image_height;
    const size_t px = (size_t)w * h;
    ok = mbgb_compile_image16_device(ctx, &sc, outs[i].image_float, w, h, img16[i]) == MBGB_OK;
    if (ok && sc.SSAOEnabled) ok = mbgb_ssao_device(ctx, &sc, &outs[i], img16[i]) == MBGB_OK;
    // the DOF shuffle draws from rand(); the reference continues its process's stream there,
    // mbgb_cli seeds it with the scene's colouring seed
    if (ok && sc.DOFEnabled) ok = mbgb_dof_device(ctx, &sc, &outs[i], img16[i], (uint32_t)sc.coloring_seed) == MBGB_OK;
    if (!ok) {
      fprintf(stderr, "mbgb_cli: post-processing: %s\n", mbgb_last_error());
      break;
    }
    host16.resize(px * 3);
    if (cudaMemcpy(host16.data(), img16[i], px * 6, cudaMemcpyDeviceToHost) != cudaSuccess) { ok = false; break; }
    mbgb_status st;
    if (a.format == kPNG16) {
      st = mbgb_write_png(jobs[i].file.c_str(), w, h, 16, 3, host16.data());
    } else if (a.format == kPNG16Alpha) {
      hostAlpha.resize(px);
      if (cudaMemcpy(hostAlpha.data(), outs[i].alpha, px * 2, cudaMemcpyDeviceToHost) != cudaSuccess) { ok = false; break; }
      std::vector<uint16_t> rgba(px * 4);
      for (size_t p = 0; p < px; p++) {
        rgba[4 * p + 0] = host16[3 * p + 0];
        rgba[4 * p + 1] = host16[3 * p + 1];
        rgba[4 * p + 2] = host16[3 * p + 2];
        rgba[4 * p + 3] = hostAlpha[p];
      }
      st = mbgb_write_png(jobs[i].file.c_str(), w, h, 16, 4, rgba.data());
    } else {
      // ConvertTo8bit (src/cimage.cpp:226-236)
      host8.resize(px * 3);
      for (size_t p = 0; p < px * 3; p++) host8[p] = (uint8_t)(host16[p] / 256);
      st = mbgb_write_png(jobs[i].file.c_str(), w, h, 8, 3, host8.data());
    }
    if (st != MBGB_OK) {
      fprintf(stderr, "mbgb_cli: %s\n", mbgb_last_error());
      ok = false;
      break;
    }
    printf("frame %d written: %s\n", jobs[i].index, jobs[i].file.c_str());
  }
  cudaFree(dev);
  return ok;
}

}  // namespace

int main(int argc, char **argv) {
  Args a;
  if (!parse(argc, argv, a)) {
    printf("commandline: wrong parameters\n");
    usage();
    return 1;
  }
  std::vector<const char *> ov;
  for (const std::string &o : a.overrides) ov.push_back(o.c_str());
  const char *defaults = a.defaults.empty() ? nullptr : a.defaults.c_str();
  mbgb_scene scene;
  if (mbgb_scene_from_settings(defaults, a.settings.c_str(), ov.data(), (int)ov.size(), &scene) != MBGB_OK) {
    fprintf(stderr, "mbgb_cli: %s\n", mbgb_last_error());
    return 1;
  }
  if (scene.noOfTiles > 1) {
    fprintf(stderr, "mbgb_cli: tiled output is not supported\n");
    return 1;
  }
  char buf[1000];
  std::string dest = "images/image";
  if (mbgb_settings_string(defaults, a.settings.c_str(), ov.data(), (int)ov.size(), "file_destination", buf,
                           sizeof(buf)) == MBGB_OK)
    dest = buf;
  const char *ext = a.format == kJPG ? "jpg" : "png";
  if (a.format == kJPG) {
    printf("mbgb_cli: no JPEG writer; writing 8-bit PNG files\n");
    ext = "png";
  }
  mbgb_context *ctx = nullptr;
  if (mbgb_context_create(a.device, &ctx) != MBGB_OK) {
    fprintf(stderr, "mbgb_cli: %s\n", mbgb_last_error());
    return 1;
  }
  std::vector<Job> pending;
  bool ok = true;
  auto flush = [&]() {
    if (ok && !pending.empty()) ok = render_jobs(ctx, pending, a);
    pending.clear();
  };
  auto add = [&](int index, const mbgb_scene &sc) {
    const std::string file = index_filename(dest, ext, index);
    if (exists(file)) {
      printf("Output file (%s) exists. Skip to next file index\n", file.c_str());
      return;
    }
    if (mbgb_scene_supported(&sc) != MBGB_OK) {
      fprintf(stderr, "mbgb_cli: frame %d: %s\n", index, mbgb_last_error());
      ok = false;
      return;
    }
    pending.push_back(Job{index, sc, file});
    if ((int)pending.size() >= a.batch) flush();
  };

  if (a.keyframe) {
    std::string keys = "keyframes/keyframe";
    if (mbgb_settings_string(defaults, a.settings.c_str(), ov.data(), (int)ov.size(), "file_keyframes", buf,
                             sizeof(buf)) == MBGB_OK)
      keys = buf;
    std::vector<mbgb_scene> keyScenes;
    for (int k = 0;; k++) {
      const std::string f = index_filename(keys, "fract", k);
      if (!exists(f)) break;
      mbgb_scene ks;
      if (mbgb_scene_from_settings(defaults, f.c_str(), ov.data(), (int)ov.size(), &ks) != MBGB_OK) {
        fprintf(stderr, "mbgb_cli: %s\n", mbgb_last_error());
        mbgb_context_destroy(ctx);
        return 1;
      }
      keyScenes.push_back(ks);
    }
    printf("Found %d keyframes\n", (int)keyScenes.size());
    const int fpk = scene.framesPerKeyframe > 0 ? scene.framesPerKeyframe : 1;
    int start = a.start > 0 ? a.start : scene.startFrame;
    int end = a.end < 99999 ? a.end : scene.endFrame;
    if (end > (int)keyScenes.size() * fpk) end = (int)keyScenes.size() * fpk;
    for (int f = start; ok && f < end; f++) {
      mbgb_scene fr;
      if (mbgb_scene_interpolate(keyScenes.data(), (int)keyScenes.size(), fpk, f, &scene, &fr) != MBGB_OK) {
        fprintf(stderr, "mbgb_cli: %s\n", mbgb_last_error());
        ok = false;
        break;
      }
      add(f, fr);
    }
  } else if (a.flight) {
    std::string pathFile = "paths/path.txt";
    if (mbgb_settings_string(defaults, a.settings.c_str(), ov.data(), (int)ov.size(), "file_animation_path", buf,
                             sizeof(buf)) == MBGB_OK)
      pathFile = buf;
    FILE *fp = fopen(pathFile.c_str(), "r");
    if (!fp) {
      fprintf(stderr, "mbgb_cli: cannot open flight path %s\n", pathFile.c_str());
      mbgb_context_destroy(ctx);
      return 1;
    }
    int start = a.start > 0 ? a.start : scene.startFrame;
    int end = a.end < 99999 ? a.end : scene.endFrame;
    for (int f = 0; ok && f < end; f++) {
      double v[6];
      if (fscanf(fp, "%lf %lf %lf %lf %lf %lf", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]) != 6) break;
      if (f < start) continue;
      mbgb_scene fr = scene;
      fr.vp[0] = v[0];
      fr.vp[1] = v[1];
      fr.vp[2] = v[2];
      fr.alpha = v[3];
      fr.beta = v[4];
      fr.gamma = v[5];
      fr.zoom = 1e-15;
      mbgb_scene_finalize(&fr);
      add(f, fr);
    }
    fclose(fp);
  } else {
    add(0, scene);
  }
  flush();
  mbgb_context_destroy(ctx);
  return ok ? 0 : 1;
}
