// TreeTrainerParameters and the TreeTrainer interface, as the reference defines
// them (tree_trainer.hpp:35-86).
#ifndef PADENTI_GB300_TREE_TRAINER_HPP
#define PADENTI_GB300_TREE_TRAINER_HPP

#include <padenti/training_set.hpp>
#include <padenti/tree.hpp>

template <typename FeatType, unsigned int FeatDim>
class TreeTrainerParameters {
 public:
  unsigned int nFeatures = 0;          // candidates sampled per node
  unsigned int nThresholds = 0;        // thresholds sampled per candidate
  bool computeFRange = false;          // unused (as in the reference)
  FeatType featLowBounds[FeatDim] = {};
  FeatType featUpBounds[FeatDim] = {};
  FeatType thrLowBound = 0;
  FeatType thrUpBound = 0;
  bool randomThrSampling = true;       // unused (as in the reference)
  unsigned int perLeafSamplesThr = 0;  // a node with at most this many samples is not split
};

template <typename ImgType, unsigned int nChannels, typename FeatType, unsigned int FeatDim, unsigned int nClasses>
class TreeTrainer {
 public:
  virtual void train(Tree<FeatType, FeatDim, nClasses> &tree, const TrainingSet<ImgType, nChannels> &trainingSet,
                     const TreeTrainerParameters<FeatType, FeatDim> &params, unsigned int startDepth,
                     unsigned int endDepth) = 0;
  virtual ~TreeTrainer() {}
};

#endif
