// Trains one tree and predicts one image through the C++ facade
// (CUDATreeTrainer / CUDAClassifier over libpadenti_gb300) on the seeded
// synthetic depth set; writes the tree XML to argv[1] and the posterior of
// image 0 (planar float32) to argv[2].  With argv[3], the feature is the user
// source at that path (compiled at run time) instead of the built-in plugin.
#include <padenti/cuda_tree_trainer.hpp>

#include <cstdio>
#include <vector>

int main(int argc, char **argv) {
  if (argc != 3 && argc != 4) return 2;
  const unsigned int n = 8, W = 160, H = 120, S = 500;
  std::vector<uint16_t> px((size_t)n * W * H);
  std::vector<uint8_t> lb((size_t)n * W * H);
  std::vector<uint32_t> sm((size_t)n * S);
  padenti_gb300::check(pd_synth_depth(0, 0, n, W, H, 1, 3, 0, S, 100, px.data(), lb.data(), sm.data()));
  std::vector<TrainingSetImage<unsigned short, 1>> imgs;
  for (unsigned int i = 0; i < n; i++)
    imgs.emplace_back(px.data() + (size_t)i * W * H, W, H, lb.data() + (size_t)i * W * H, 3,
                      sm.data() + (size_t)i * S, S);
  TrainingSet<unsigned short, 1> ts(3, imgs);
  TreeTrainerParameters<int, 4> p;
  p.nFeatures = 64;
  p.nThresholds = 20;
  for (int d = 0; d < 4; d++) {
    p.featLowBounds[d] = -60000;
    p.featUpBounds[d] = 60000;
  }
  p.thrLowBound = -500;
  p.thrUpBound = 500;
  p.perLeafSamplesThr = 20;
  Tree<int, 4, 3> tree(3, 7);
  using Trainer = CUDATreeTrainer<unsigned short, 1, int, 4, 3>;
  using Clf = CUDAClassifier<unsigned short, 1, int, 4, 3>;
  Trainer trainer = argc == 4 ? Trainer(std::string(argv[3])) : Trainer(PD_PLUGIN_DEPTH_DIFF2);
  trainer.train(tree, ts, p, 1, 7);
  tree.save(argv[1]);
  Clf clf = argc == 4 ? Clf(std::string(argv[3])) : Clf(PD_PLUGIN_DEPTH_DIFF2);
  clf << tree;
  Image<unsigned short, 1> image(px.data(), W, H);
  Image<float, 3> post(W, H);
  clf.predict(image, post);
  FILE *f = std::fopen(argv[2], "wb");
  if (!f) return 4;
  std::fwrite(post.getData(), sizeof(float), (size_t)3 * W * H, f);
  std::fclose(f);
  return 0;
}
