// Samples seeded synthetic depth maps through the C++ sampler facade
// (CUDAUniformImageSampler, CUDAClassWeightedImageSampler), one image at a time
// through sample() and all at once through sampleBatch(), and builds a
// TrainingSet with sampledTrainingSet(); writes, as uint32: for each of the
// three runs and each image, the count then the samples, to argv[1].
#include <padenti/cuda_tree_trainer.hpp>
#include <padenti/image_sampler.hpp>

#include <algorithm>
#include <cstdio>
#include <vector>

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  const unsigned int n = 4, W = 160, H = 120;
  std::vector<uint16_t> px((size_t)n * W * H);
  std::vector<uint8_t> lb((size_t)n * W * H);
  std::vector<uint32_t> unused((size_t)n);
  padenti_gb300::check(pd_synth_depth(4, 0, n, W, H, 1, 3, 0, 1, 100, px.data(), lb.data(), unused.data()));
  std::vector<uint32_t> out;
  CUDAUniformImageSampler<unsigned short, 1> uni(500, 3);
  const float w[3] = {0.5f, 0.25f, 0.3f};
  CUDAClassWeightedImageSampler<unsigned short, 1> cw(400, 3, w, 7);
  std::vector<unsigned int> buf(std::max(uni.gpu().stride(), cw.gpu().stride()));
  for (unsigned int i = 0; i < n; i++) {
    const unsigned int c = uni.sample(px.data() + (size_t)i * W * H, lb.data() + (size_t)i * W * H, W, H, buf.data());
    out.push_back(c);
    out.insert(out.end(), buf.begin(), buf.begin() + c);
  }
  std::vector<const unsigned short *> d;
  std::vector<const unsigned char *> l;
  for (unsigned int i = 0; i < n; i++) {
    d.push_back(px.data() + (size_t)i * W * H);
    l.push_back(lb.data() + (size_t)i * W * H);
  }
  const unsigned int stride = cw.gpu().stride();
  std::vector<unsigned int> all((size_t)n * stride);
  const std::vector<unsigned int> cnt = cw.gpu().sampleBatch(d, l, std::vector<unsigned int>(n, W),
                                                             std::vector<unsigned int>(n, H), all.data());
  for (unsigned int i = 0; i < n; i++) {
    out.push_back(cnt[i]);
    out.insert(out.end(), all.begin() + (size_t)i * stride, all.begin() + (size_t)i * stride + cnt[i]);
  }
  std::vector<Image<unsigned short, 1>> imgs;
  std::vector<Image<unsigned char, 1>> labs;
  for (unsigned int i = 0; i < n; i++) {
    imgs.emplace_back(d[i], W, H);
    labs.emplace_back(l[i], W, H);
  }
  const TrainingSet<unsigned short, 1> ts = sampledTrainingSet(3, imgs, labs, cw, stride);
  for (const auto &im : ts.getImages()) {
    out.push_back(im.getNSamples());
    out.insert(out.end(), im.getSamples(), im.getSamples() + im.getNSamples());
  }
  FILE *f = std::fopen(argv[1], "wb");
  if (!f) return 4;
  std::fwrite(out.data(), 4, out.size(), f);
  std::fclose(f);
  return 0;
}
