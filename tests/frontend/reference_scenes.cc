// Driver for the reference's own scene functions (src/utils.cc: random_scene
// ... oneweek_final), compiled unchanged against include/tpt_scene.hpp.  The
// functions' text is not part of this repository: tests/test_frontend.py
// copies it from a reference checkout into reference_scene_functions.inc in
// a temporary directory at test time.
//
// Usage: reference_scenes <function>.  Builds the scene, compiles it, and
// prints every bvh_node the function created, in creation order: a line
// "tree <nodes>", then per node in pre-order its box (6 floats) and its two
// children (pre-order index, or -1 for a leaf).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tpt_scene.hpp"

using namespace tpt;

// stb_image's loader as the reference's image scenes call it
// (utils.cc:236-240,400): no file is read; a 16 x 8 RGB gradient stands in.
static unsigned char *stbi_load(const char *, int *x, int *y, int *comp, int) {
  static unsigned char px[16 * 8 * 3];
  for (int i = 0; i < 16 * 8; i++) {
    px[3 * i] = (unsigned char)(16 * (i % 16));
    px[3 * i + 1] = (unsigned char)(32 * (i / 16));
    px[3 * i + 2] = 128;
  }
  *x = 16;
  *y = 8;
  *comp = 3;
  return px;
}

hitable *two_checker_spheres();
hitable *random_scene();
hitable *two_perlin_spheres();
hitable *light_spheres();
hitable *sphere_cornell_box();
hitable *cornell_box();
hitable *cornell_box_smoke();
hitable *oneweek_final();

#include "reference_scene_functions.inc"

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  const std::string name = argv[1];
  struct {
    const char *name;
    hitable *(*fn)();
  } table[] = {{"random_scene", random_scene},           {"two_checker_spheres", two_checker_spheres},
               {"two_perlin_spheres", two_perlin_spheres}, {"light_spheres", light_spheres},
               {"sphere_cornell_box", sphere_cornell_box}, {"cornell_box", cornell_box},
               {"cornell_box_smoke", cornell_box_smoke},   {"oneweek_final", oneweek_final}};
  hitable *(*fn)() = nullptr;
  for (const auto &e : table)
    if (name == e.name) fn = e.fn;
  if (!fn) return 2;
  hitable *world = fn();
  camera cam(vec3(0, 0, 800), vec3(0, 0, 0), vec3(0, 1, 0), 40, 1, 0, 10, 0, 1);
  tpt_scene *s = compile_scene(world, nullptr, cam);
  for (int32_t h = 0; h < (1 << 18); h++) {
    const int32_t n = tpt_scene_bvh_dump(s, h, nullptr, nullptr, 0);
    if (n <= 0) continue;
    std::vector<float> boxes(6 * (size_t)n);
    std::vector<int32_t> kids(2 * (size_t)n);
    tpt_scene_bvh_dump(s, h, boxes.data(), kids.data(), n);
    std::printf("tree %d\n", n);
    for (int i = 0; i < n; i++) {
      const float *b = &boxes[6 * (size_t)i];
      std::printf("%.9g %.9g %.9g %.9g %.9g %.9g %d %d\n", b[0], b[1], b[2], b[3], b[4], b[5],
                  kids[2 * i] < 0 ? -1 : kids[2 * i], kids[2 * i + 1] < 0 ? -1 : kids[2 * i + 1]);
    }
  }
  tpt_scene_destroy(s);
  return 0;
}
