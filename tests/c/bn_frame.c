/* bn_frame.c -- one frame through the barney-compatible bn* API from plain C:
   a 33^3 field built from host texels, a 16-entry transfer function, one
   directional light, a perspective camera, 4 paths per pixel at 64x48;
   writes the FLOAT4 frame (64*48*4 floats) to argv[1]. */
#include <stdio.h>
#include <stdlib.h>
#include "barney_gb300.h"

#define N 33
#define W 64
#define H 48

int main(int argc, char **argv) {
  static float voxels[N * N * N];
  static float tf[16 * 4];
  static float frame[W * H * 4];
  int i, j, k;
  BNContext ctx;
  BNTextureData td;
  BNScalarField sf;
  BNVolume vol;
  BNLight light;
  BNData lights;
  BNGroup grp;
  BNModel model;
  BNCamera cam;
  BNRenderer ren;
  BNFrameBuffer fb;
  bn_float2 domain = {0.f, 1.f};
  FILE *f;
  if (argc < 2) return 2;
  for (k = 0; k < N; k++)
    for (j = 0; j < N; j++)
      for (i = 0; i < N; i++) voxels[i + N * (j + N * k)] = (float)((i * 7 + j * 13 + k * 29) % 97) / 96.0f;
  for (i = 0; i < 16; i++) {
    tf[4 * i + 0] = (float)i / 15.0f;
    tf[4 * i + 1] = 0.5f;
    tf[4 * i + 2] = 1.0f - (float)i / 15.0f;
    tf[4 * i + 3] = (float)i / 15.0f * 0.8f;
  }
  ctx = bnContextCreate(0, 1, 0, -1);
  if (!ctx) { fprintf(stderr, "context: %s\n", bnGetLastError()); return 1; }
  td = bnTextureData3DCreate(ctx, 0, BN_FLOAT, N, N, N, voxels);
  sf = bnScalarFieldCreate(ctx, 0, "structured");
  bnSetObject(sf, "textureData", td);
  bnSet3i(sf, "dims", N, N, N);
  bnSet3f(sf, "gridOrigin", -0.5f, -0.5f, -0.5f);
  bnSet3f(sf, "gridSpacing", 0.03125f, 0.03125f, 0.03125f);
  bnCommit(sf);
  vol = bnVolumeCreate(ctx, 0, sf);
  bnVolumeSetXF(vol, domain, (const bn_float4 *)tf, 16, 10.f);
  bnCommit(vol);
  light = bnLightCreate(ctx, 0, "directional");
  bnSet3f(light, "direction", -1.f, -1.f, -1.f);
  bnSet3f(light, "color", 1.f, 1.f, 1.f);
  bnSet1f(light, "radiance", 2.f);
  bnCommit(light);
  lights = bnDataCreate(ctx, 0, BN_OBJECT, 1, &light);
  grp = bnGroupCreate(ctx, 0, 0, 0, &vol, 1);
  bnSetData(grp, "lights", lights);
  bnCommit(grp);
  bnGroupBuild(grp);
  model = bnModelCreate(ctx);
  bnSetInstances(model, 0, &grp, 0, 1);
  bnBuild(model, 0);
  cam = bnCameraCreate(ctx, "perspective");
  bnSet3f(cam, "position", 0.5f, 0.625f, 2.25f);
  bnSet3f(cam, "direction", -0.5f, -0.625f, -2.25f);
  bnSet3f(cam, "up", 0.f, 1.f, 0.f);
  bnSet1f(cam, "fovy", 40.f);
  bnCommit(cam);
  ren = bnRendererCreate(ctx, "default");
  bnSet1i(ren, "pathsPerPixel", 4);
  bnSet1f(ren, "ambientRadiance", 0.25f);
  bnSet4f(ren, "bgColor", 0.f, 0.f, 0.f, 1.f);
  bnCommit(ren);
  fb = bnFrameBufferCreate(ctx, 0);
  bnFrameBufferResize(fb, BN_FLOAT4, W, H, BN_FB_COLOR);
  bnRender(ren, model, cam, fb);
  bnFrameBufferRead(fb, BN_FB_COLOR, frame, BN_FLOAT4);
  if (bnGetLastError()[0]) { fprintf(stderr, "bn: %s\n", bnGetLastError()); return 1; }
  f = fopen(argv[1], "wb");
  if (!f || fwrite(frame, sizeof(float), W * H * 4, f) != (size_t)(W * H * 4)) return 3;
  fclose(f);
  bnContextDestroy(ctx);
  printf("frame written\n");
  return 0;
}
