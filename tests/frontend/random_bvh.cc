// Scene code in the reference's style, compiled against include/tpt_scene.hpp:
// n spheres whose layout is drawn with drand_r, then one bvh_node over them.
// Prints the BVH's node boxes in pre-order, one node per line (6 floats).
// Used by tests/test_frontend.py.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tpt_scene.hpp"

using namespace tpt;

int main(int argc, char **argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 100;
  material *m = new lambertian(new constant_texture(vec3(0.5f, 0.5f, 0.5f)));
  std::vector<hitable *> list;
  for (int i = 0; i < n; i++) {
    const float x = (float)drand_r(-10, 10);
    const float z = (float)drand_r(-10, 10);
    const float r = (float)(0.1 + 0.3 * drand_r());
    list.push_back(new sphere(vec3(x, r, z), r, m));
  }
  hitable *world = new bvh_node(list.data(), n, 0.0f, 1.0f);
  camera_with_blur cam(vec3(13, 2, 3), vec3(0, 0, 0), vec3(0, 1, 0), 20, 1.5f, 0.1f, 10, 0, 1);
  tpt_scene *s = compile_scene(world, nullptr, cam);
  const int nodes = tpt_scene_bvh_dump(s, world->handle, nullptr, nullptr, 0);
  if (nodes < 0) return 2;
  std::vector<float> boxes(6 * (size_t)nodes);
  std::vector<int32_t> kids(2 * (size_t)nodes);
  tpt_scene_bvh_dump(s, world->handle, boxes.data(), kids.data(), nodes);
  for (int i = 0; i < nodes; i++)
    std::printf("%.9g %.9g %.9g %.9g %.9g %.9g\n", boxes[6 * i], boxes[6 * i + 1], boxes[6 * i + 2], boxes[6 * i + 3],
                boxes[6 * i + 4], boxes[6 * i + 5]);
  tpt_scene_destroy(s);
  return 0;
}
