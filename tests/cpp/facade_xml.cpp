// Tree XML round trip through the C++ facade (no GPU): loads the tree file given
// as argv[1] (tree id argv[2]), checks the heap invariants, and saves it again to
// argv[3].  The test compares the saved text with the input.
#include <padenti/tree.hpp>
#include <padenti/training_set.hpp>

#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  Tree<int, 4, 3> tree;
  tree.load(argv[1], std::atoi(argv[2]));
  for (size_t i = 0; i < tree.getNNodes(); i++) {
    const int c = tree.getLeftChildren()[i];
    if (c >= 0 && (size_t)c != 2 * i + 1) return 3;
  }
  tree.save(argv[3]);
  // priors of a two-image set built both ways
  unsigned short px[4] = {1, 2, 3, 4};
  unsigned char lab[4] = {1, 2, 2, 0};
  unsigned int sm[3] = {0, 1, 2};
  TrainingSetImage<unsigned short, 1> a(px, 2, 2, lab, 3, sm, 3);
  unsigned int sm2[2] = {1, 1};
  TrainingSetImage<unsigned short, 1> b(px, 2, 2, lab, 3, sm2, 2);
  TrainingSet<unsigned short, 1> mean(3, {a, b});
  TrainingSet<unsigned short, 1> inc(3);
  inc << a << b;
  std::printf("%.9g %.9g %.9g | %.9g %.9g %.9g\n", mean.getPriors()[0], mean.getPriors()[1], mean.getPriors()[2],
              inc.getPriors()[0], inc.getPriors()[1], inc.getPriors()[2]);
  return 0;
}
