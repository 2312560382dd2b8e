// Loads the PGM argv[1] through PNMImageROILoader (both load() forms) and prints
// the cropped size, the crop's corner and the first cropped pixel of each.
#include <padenti/image_loader.hpp>

#include <cstdio>
#include <vector>

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  PNMImageROILoader<unsigned short, 1> loader;
  const Image<unsigned short, 1> im = loader.load(argv[1]);
  std::printf("%u %u %u %u %u\n", im.getWidth(), im.getHeight(), loader.getRoiX(), loader.getRoiY(),
              (unsigned)im.getData()[0]);
  const padenti_gb300::Pnm p = padenti_gb300::read_pnm(argv[1]);
  std::vector<unsigned short> buf((size_t)p.width * p.height);
  unsigned int w = 0, h = 0;
  loader.load(argv[1], buf.data(), &w, &h);
  std::printf("%u %u %u %u %u\n", w, h, loader.getRoiX(), loader.getRoiY(), (unsigned)buf[0]);
  return 0;
}
