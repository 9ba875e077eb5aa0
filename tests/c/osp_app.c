/* A small OSPRay application written against include/ospray (C99), used by
 * the tests to check that an unmodified API client builds, links and renders
 * through libospray.so + the b200 device module.
 *
 * It renders two coloured triangles under an ambient light with the path
 * tracer into an sRGB framebuffer, first one frame and then ten accumulated
 * frames, writes both as binary PPM, picks the centre of the screen, and
 * prints one line of results: "bounds x0 y0 z0 x1 y1 z1 pick hit prim mean0
 * mean10 duration".  Exit status: 0 on success, the OSPError otherwise. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "ospray/ospray_util.h"

static int g_errors = 0;

static void onError(void *user, OSPError e, const char *msg) {
  (void)user;
  fprintf(stderr, "OSPRay error %d: %s\n", (int)e, msg);
  g_errors++;
}

static double meanAndWrite(const char *path, int w, int h, const uint32_t *px) {
  FILE *f = fopen(path, "wb");
  double sum = 0.0;
  if (f) fprintf(f, "P6\n%d %d\n255\n", w, h);
  for (int y = h - 1; y >= 0; y--) /* rows are stored bottom-up */
    for (int x = 0; x < w; x++) {
      const uint32_t p = px[(size_t)y * w + x];
      const unsigned char rgb[3] = {(unsigned char)(p & 255), (unsigned char)((p >> 8) & 255),
                                    (unsigned char)((p >> 16) & 255)};
      sum += rgb[0] + rgb[1] + rgb[2];
      if (f) fwrite(rgb, 1, 3, f);
    }
  if (f) fclose(f);
  return sum / (3.0 * w * h);
}

int main(int argc, const char **argv) {
  const int W = 320, H = 240;
  const char *outdir = argc > 1 ? argv[1] : ".";
  char path[1024];

  OSPError err = ospInit(&argc, argv);
  if (err != OSP_NO_ERROR) {
    fprintf(stderr, "ospInit failed: %s\n", ospDeviceGetLastErrorMsg(NULL));
    return (int)err;
  }
  OSPDevice dev = ospGetCurrentDevice();
  ospDeviceSetErrorCallback(dev, onError, NULL);
  ospDeviceRelease(dev);

  /* camera */
  float pos[] = {0.f, 0.f, 0.f}, up[] = {0.f, 1.f, 0.f}, dir[] = {0.1f, 0.f, 1.f};
  OSPCamera camera = ospNewCamera("perspective");
  ospSetFloat(camera, "aspect", W / (float)H);
  ospSetParam(camera, "position", OSP_VEC3F, pos);
  ospSetParam(camera, "direction", OSP_VEC3F, dir);
  ospSetParam(camera, "up", OSP_VEC3F, up);
  ospCommit(camera);

  /* two triangles (a quad split along its diagonal), per-vertex colours */
  float vertex[] = {-1.f, -1.f, 3.f, -1.f, 1.f, 3.f, 1.f, -1.f, 3.f, 0.1f, 0.1f, 0.3f};
  float color[] = {0.9f, 0.5f, 0.5f, 1.f, 0.8f, 0.8f, 0.8f, 1.f, 0.8f, 0.8f, 0.8f, 1.f, 0.5f, 0.9f, 0.5f, 1.f};
  int32_t index[] = {0, 1, 2, 1, 2, 3};
  OSPGeometry mesh = ospNewGeometry("mesh");
  OSPData d = ospNewSharedData1D(vertex, OSP_VEC3F, 4);
  ospCommit(d);
  ospSetObject(mesh, "vertex.position", d);
  ospRelease(d);
  d = ospNewSharedData1D(color, OSP_VEC4F, 4);
  ospCommit(d);
  ospSetObject(mesh, "vertex.color", d);
  ospRelease(d);
  d = ospNewSharedData1D(index, OSP_VEC3UI, 2);
  ospCommit(d);
  ospSetObject(mesh, "index", d);
  ospRelease(d);
  ospCommit(mesh);

  OSPMaterial mat = ospNewMaterial("obj");
  ospCommit(mat);
  OSPGeometricModel model = ospNewGeometricModel(mesh);
  ospSetObject(model, "material", mat);
  ospCommit(model);
  ospRelease(mesh);
  ospRelease(mat);

  OSPGroup group = ospNewGroup();
  ospSetObjectAsData(group, "geometry", OSP_GEOMETRIC_MODEL, model);
  ospCommit(group);
  ospRelease(model);
  OSPInstance instance = ospNewInstance(group);
  ospCommit(instance);
  ospRelease(group);

  OSPWorld world = ospNewWorld();
  ospSetObjectAsData(world, "instance", OSP_INSTANCE, instance);
  ospRelease(instance);
  OSPLight light = ospNewLight("ambient");
  ospCommit(light);
  ospSetObjectAsData(world, "light", OSP_LIGHT, light);
  ospRelease(light);
  ospCommit(world);
  OSPBounds b = ospGetBounds(world);

  OSPRenderer renderer = ospNewRenderer("pathtracer");
  ospSetFloat(renderer, "backgroundColor", 1.0f);
  ospCommit(renderer);

  OSPFrameBuffer fb = ospNewFrameBuffer(W, H, OSP_FB_SRGBA, OSP_FB_COLOR | OSP_FB_ACCUM);
  ospResetAccumulation(fb);

  ospRenderFrameBlocking(fb, renderer, camera, world);
  const uint32_t *px = (const uint32_t *)ospMapFrameBuffer(fb, OSP_FB_COLOR);
  snprintf(path, sizeof(path), "%s/firstFrame.ppm", outdir);
  const double mean0 = px ? meanAndWrite(path, W, H, px) : -1.0;
  ospUnmapFrameBuffer(px, fb);

  float duration = 0.f;
  for (int i = 0; i < 10; i++) {
    OSPFuture fut = ospRenderFrame(fb, renderer, camera, world);
    ospWait(fut, OSP_TASK_FINISHED);
    if (!ospIsReady(fut, OSP_TASK_FINISHED)) g_errors++;
    duration += ospGetTaskDuration(fut);
    ospRelease(fut);
  }
  px = (const uint32_t *)ospMapFrameBuffer(fb, OSP_FB_COLOR);
  snprintf(path, sizeof(path), "%s/accumulatedFrame.ppm", outdir);
  const double mean10 = px ? meanAndWrite(path, W, H, px) : -1.0;
  ospUnmapFrameBuffer(px, fb);

  OSPPickResult p;
  ospPick(&p, fb, renderer, camera, world, 0.5f, 0.5f);
  printf("bounds %g %g %g %g %g %g pick %d %u mean0 %.3f mean10 %.3f duration %.6f\n", b.lower[0], b.lower[1],
         b.lower[2], b.upper[0], b.upper[1], b.upper[2], p.hasHit, p.primID, mean0, mean10, duration);
  ospRelease(p.instance);
  ospRelease(p.model);
  ospRelease(renderer);
  ospRelease(camera);
  ospRelease(fb);
  ospRelease(world);
  ospShutdown();
  return g_errors ? 1 : 0;
}
