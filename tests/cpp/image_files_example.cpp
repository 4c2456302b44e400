// ImageTexture(filename, flip_y, isHDR) and EnvironmentLight(hdri_filepath)
// as a reference scene would construct them: prints the width, height and
// texels of each, one value per line.
#include <cstdio>
#include <string>

#include "pathtracer_gb300.hpp"

using namespace ptgb;

static void dump(const std::vector<float> &t, int w, int h) {
  std::printf("%d %d\n", w, h);
  for (float v : t) std::printf("%.9g\n", v);
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  ImageTexture png(argv[1], /*flip_y=*/true);
  dump(png.texels, png.width, png.height);
  EnvironmentLight env(argv[2], 2.0f);
  dump(env.texels, env.width, env.height);
  try {
    ImageTexture missing(std::string(argv[1]) + ".missing");
  } catch (const std::runtime_error &) {
    std::printf("missing-file error\n");
  }
  return 0;
}
