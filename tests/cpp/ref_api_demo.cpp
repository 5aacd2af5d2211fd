// ref_api_demo.cpp -- drives libkdgr through the reference's own C++ call
// sequence (renderingTestInit + one frame, Kd-treeConverterMain.cpp:3618-3651
// and :3548): read the .kdt, invert the scales as the reference caller does,
// set up, render one frame into a device framebuffer, write it to a file.
//
// A scene given as .ply goes through loadGaussiansFromPly.
//
// usage: ref_api_demo scene.(kdgs|ply) tree.kdt W H px py pz ux uy uz vx vy vz nx ny nz fovy aspect near out.bin
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "kdgr_reference_api.h"

static bool read_kdgs(const char* path, std::vector<Gaussian>& out) {
  FILE* fp = fopen(path, "rb");
  if (!fp) return false;
  char magic[4];
  unsigned hdr[3];
  bool ok = fread(magic, 1, 4, fp) == 4 && memcmp(magic, "KDGS", 4) == 0 && fread(hdr, 4, 3, fp) == 3 &&
            hdr[0] == 1 && hdr[2] == 64;
  if (ok) {
    out.resize(hdr[1]);
    ok = fread(out.data(), sizeof(Gaussian), hdr[1], fp) == hdr[1];
  }
  fclose(fp);
  return ok;
}

int main(int argc, char** argv) {
  if (argc != 21) {
    fprintf(stderr, "usage: %s scene.kdgs tree.kdt W H pos(3) u(3) v(3) n(3) fovy aspect near out.bin\n", argv[0]);
    return 2;
  }
  std::vector<Gaussian> gaussians;
  const size_t len = strlen(argv[1]);
  const bool ply = len > 4 && strcmp(argv[1] + len - 4, ".ply") == 0;
  if (!(ply ? loadGaussiansFromPly(argv[1], gaussians) : read_kdgs(argv[1], gaussians))) return 3;
  CompositeObject obj;
  memset(&obj, 0, sizeof(obj));
  if (!read_kd_tree_from_file(&obj, argv[2], KD_TREE_DUMP_IN_BINARY)) return 4;
  for (Gaussian& g : gaussians) {  // the caller-side inversion (Kd-treeConverterMain.cpp:3636-3650)
    g.scale[0] = 1 / g.scale[0];
    g.scale[1] = 1 / g.scale[1];
    g.scale[2] = 1 / g.scale[2];
    g.k_scale = 1 / g.k_scale;
  }
  if (!initCuda()) return 5;
  // KDGR_DEMO_SECONDARY=sphere|tri: the SECONDARY_RAY build's setup with a
  // mirror square behind the scene (SecondaryMesh defaults), rendering
  // against the demo spheres or that mesh
  const char* sec = getenv("KDGR_DEMO_SECONDARY");
  if (sec && (!strcmp(sec, "sphere") || !strcmp(sec, "tri"))) {
    SecondaryMesh mesh;
    const float3 a = {-0.9f, -0.9f, -0.6f}, b = {0.9f, -0.9f, -0.6f}, c = {0.9f, 0.9f, -0.6f}, d = {-0.9f, 0.9f, -0.6f};
    mesh.vert = {a, b, c, a, c, d};
    mesh.triangleCount = 2;
    renderGaussianWithCudaSetup(obj, gaussians, mesh);
    setSecondaryPrimitive(!strcmp(sec, "tri") ? KDGR_SECONDARY_TRI : KDGR_SECONDARY_SPHERE);
  } else {
    renderGaussianWithCudaSetup(obj, gaussians);
  }
  const int W = atoi(argv[3]), H = atoi(argv[4]);
  Camera cam;
  memset(&cam, 0, sizeof(cam));
  for (int i = 0; i < 3; ++i) {
    cam.pos[i] = (float)atof(argv[5 + i]);
    cam.uaxis[i] = (float)atof(argv[8 + i]);
    cam.vaxis[i] = (float)atof(argv[11 + i]);
    cam.naxis[i] = (float)atof(argv[14 + i]);
  }
  cam.fovy = atof(argv[17]);
  cam.aspect = atof(argv[18]);
  cam.near_c = atof(argv[19]);
  float* d_fb = nullptr;
  if (cudaMalloc(&d_fb, sizeof(float) * 3 * W * H) != cudaSuccess) return 6;
  cudaMemset(d_fb, 0, sizeof(float) * 3 * W * H);
  const float fps = renderGaussianWithCudaFrame(cam, W, H, d_fb, 0);
  warmUp(d_fb, 0);
  std::vector<float> fb(3 * (size_t)W * H);
  if (cudaMemcpy(fb.data(), d_fb, fb.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
  FILE* fp = fopen(argv[20], "wb");
  if (!fp) return 8;
  fwrite(fb.data(), 4, fb.size(), fp);
  fclose(fp);
  cudaFree(d_fb);
  cleanupCudaResources();
  printf("fps %f\n", fps);
  return fps > 0.f ? 0 : 9;
}
