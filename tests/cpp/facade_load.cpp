// Loads a training set from the directory argv[1] through the C++ loader
// facade (PNMImageLoader, CUDARGBLabelsLoader, loadTrainingSet with a
// CUDAClassWeightedImageSampler(300, 3, seed 11)); writes, as uint32 per image:
// width, height, the labels (one per word), the sample count and the samples, to argv[2].
#include <padenti/image_loader.hpp>

#include <cstdio>
#include <vector>

static const unsigned char RGB2LABEL[][3] = {{255, 0, 0}, {0, 0, 255}, {0, 255, 0}};

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  PNMImageLoader<unsigned short, 1> depth;
  CUDARGBLabelsLoader labels(RGB2LABEL, 3);
  CUDAClassWeightedImageSampler<unsigned short, 1> sampler(300, 3, 11);
  const TrainingSet<unsigned short, 1> ts =
      loadTrainingSet(argv[1], "_depth.pgm", "_labels.ppm", 3, depth, labels, sampler, sampler.gpu().stride());
  std::vector<uint32_t> out;
  for (const auto &im : ts.getImages()) {
    out.push_back(im.getWidth());
    out.push_back(im.getHeight());
    for (size_t p = 0; p < (size_t)im.getWidth() * im.getHeight(); p++) out.push_back(im.getLabels()[p]);
    out.push_back(im.getNSamples());
    out.insert(out.end(), im.getSamples(), im.getSamples() + im.getNSamples());
  }
  FILE *f = std::fopen(argv[2], "wb");
  if (!f) return 4;
  std::fwrite(out.data(), 4, out.size(), f);
  std::fclose(f);
  return 0;
}
