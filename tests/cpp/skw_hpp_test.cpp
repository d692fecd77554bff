// Client of include/skw.hpp as a C++ renderer would use it: accelerator
// queries with known answers, a photon k-NN against brute force, a
// direct-lighting render and a photon shoot.  Prints "skw.hpp: OK" and
// exits 0, or prints the failed check and exits 1.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "skw.hpp"

#define EXPECT(c)                                                  \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);   \
      return 1;                                                    \
    }                                                              \
  } while (0)

static skw::Mesh square(float z, float half, bool up) {
  skw::Mesh m;
  m.vertices = {-half, -half, z, half, -half, z, half, half, z, -half, half, z};
  m.triangles = up ? std::vector<int32_t>{0, 1, 2, 0, 2, 3} : std::vector<int32_t>{0, 2, 1, 0, 3, 2};
  return m;
}

static skw_ray ray(float ox, float oy, float oz, float dx, float dy, float dz, float tmin, float tmax) {
  return skw_ray{ox, oy, oz, dx, dy, dz, tmin, tmax};
}

int main() {
  try {
    skw::Context ctx(0);

    // Two squares: mesh 0 at z = 1, mesh 1 at z = 2 moved by x + 10.
    const double shift[16] = {1, 0, 0, 10, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::vector<skw::Mesh> meshes = {square(1.0f, 1.0f, true), square(2.0f, 1.0f, true)};
    std::vector<skw_primitive> prims = {{0, nullptr}, {1, shift}};
    skw::TriangleAccelerator acc(ctx, meshes, prims);
    const float inf = INFINITY;
    std::vector<skw_ray> rays = {ray(0.1f, 0.2f, 0, 0, 0, 1, 0, inf), ray(10.1f, -0.3f, 0, 0, 0, 1, 0, inf),
                                 ray(5, 5, 0, 0, 0, 1, 0, inf), ray(-0.5f, 0.5f, 3, 0, 0, -1, 0, inf)};
    std::vector<skw_hit> hits = acc.Intersect(rays);
    EXPECT(hits[0].prim == 0 && std::fabs(hits[0].t - 1.0f) < 1e-6f);
    EXPECT(hits[1].prim == 1 && std::fabs(hits[1].t - 2.0f) < 1e-6f);
    EXPECT(hits[2].prim == -1 && std::isinf(hits[2].t));
    EXPECT(hits[3].prim == 0 && std::fabs(hits[3].t - 2.0f) < 1e-6f);
    std::vector<skw_ray> shadow = {ray(0.1f, 0.2f, 0, 0, 0, 1, 0, 0.5f), ray(0.1f, 0.2f, 0, 0, 0, 1, 0, 1.5f)};
    std::vector<uint8_t> occ = acc.IntersectTest(shadow);
    EXPECT(occ[0] == 0 && occ[1] == 1);
    EXPECT(acc.Info().n_triangles == 4);

    // k nearest of a 10 x 10 x 10 lattice (jittered) against brute force.
    std::vector<float> pos;
    for (int i = 0; i < 1000; ++i) {
      pos.push_back((float)(i % 10) + 0.01f * (float)((i * 7) % 13));
      pos.push_back((float)((i / 10) % 10) + 0.01f * (float)((i * 11) % 17));
      pos.push_back((float)(i / 100) + 0.01f * (float)((i * 5) % 19));
    }
    skw::PhotonKDTree tree(ctx, pos, std::vector<uint16_t>(1000, 0));
    const std::vector<double> q = {4.3, 5.6, 2.2};
    const int k = 8;
    skw::PhotonKDTree::Neighbours nb = tree.GetNearestPoints(q, {}, k, 2.0, -1.0);
    EXPECT(nb.count[0] == k);
    std::vector<int32_t> perm = tree.Permutation();
    std::vector<double> want;
    for (int i = 0; i < 1000; ++i) {
      double d2 = 0;
      for (int c = 0; c < 3; ++c) d2 += ((double)pos[3 * i + c] - q[c]) * ((double)pos[3 * i + c] - q[c]);
      want.push_back(d2);
    }
    std::vector<double> got;
    for (int j = 0; j < k; ++j) {
      const int orig = perm[(size_t)nb.idx[(size_t)j]];
      EXPECT(nb.d2[(size_t)j] == want[(size_t)orig]);
      got.push_back(nb.d2[(size_t)j]);
    }
    std::sort(got.begin(), got.end());
    std::sort(want.begin(), want.end());
    for (int j = 0; j < k; ++j) EXPECT(got[(size_t)j] == want[(size_t)j]);

    // Direct lighting: a matte floor under a quad light, 8 x 8, 2 x 2 spp.
    std::vector<skw::Mesh> rm = {square(0.0f, 5.0f, true), square(1.0f, 0.3f, false)};
    skw_render_primitive floor_p{0, nullptr, 0, nullptr, nullptr, {0, 0, 0}, nullptr, nullptr};
    skw_render_primitive light_p{1, nullptr, 1, nullptr, nullptr, {10, 10, 10}, nullptr, nullptr};
    skw_material matte{};
    matte.kind = SKW_MATERIAL_MATTE;
    matte.kd[0] = matte.kd[1] = matte.kd[2] = 0.5f;
    matte.roughness = 0.1f;
    skw_material black = matte;
    black.kd[0] = black.kd[1] = black.kd[2] = 0.0f;
    skw::Scene scene(ctx, rm, {floor_p, light_p}, {matte, black}, {});
    skw_camera cam{};
    // camera at (0, 0, 0.8) looking down (-z): x -> image right, y -> image down
    const double c2w[16] = {1, 0, 0, 0, 0, -1, 0, 0, 0, 0, -1, 0.8, 0, 0, 0, 1};
    std::copy(c2w, c2w + 16, cam.camera_to_world);
    cam.x_view_angle = 1.0;
    cam.width = cam.height = 8;
    skw_render_params rp{2, 2, 1, 7, SKW_SAMPLER_STRATIFIED};
    float *d_film = nullptr;
    EXPECT(cudaMalloc((void **)&d_film, 8 * 8 * 3 * sizeof(float)) == cudaSuccess);
    scene.RenderDirect(cam, rp, d_film, nullptr);
    std::vector<float> film(8 * 8 * 3);
    EXPECT(cudaMemcpy(film.data(), d_film, film.size() * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess);
    double sum = 0.0;
    for (float v : film) {
      EXPECT(std::isfinite(v) && v >= 0.0f);
      sum += v;
    }
    // the floor below a radiance-10 light of 0.36 at height 1: about
    // 0.5 / pi * 10 * 0.36 = 0.57 straight below, less towards the edges
    EXPECT(sum / film.size() > 0.2 && sum / film.size() < 0.8);

    // Photon shooting from the same light.
    skw_photon_params pp{100000, 8, 0.0f, 3};
    skw::PhotonMap pm = skw::PhotonMap::Shoot(scene, pp);
    const skw_photon_map_info info = pm.Info();
    EXPECT(info.n_direct > 50000 && info.paths_direct == 100000);
    skw_photon_render_params gp{4, 50, 0.1};
    pm.Render(scene, cam, rp, gp, d_film, nullptr);
    EXPECT(cudaDeviceSynchronize() == cudaSuccess);
    cudaFree(d_film);

    // Errors surface as skw::Error with the status code.
    bool threw = false;
    try {
      scene.SetMaxSpecularDepth(99);
    } catch (const skw::Error &e) {
      threw = e.code() == SKW_ERR_ARG;
    }
    EXPECT(threw);
    std::printf("skw.hpp: OK (launches %lld)\n", (long long)ctx.LaunchCount());
    return 0;
  } catch (const std::exception &e) {
    std::printf("FAILED: exception %s\n", e.what());
    return 1;
  }
}
