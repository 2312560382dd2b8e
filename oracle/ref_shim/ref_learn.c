/*
 * Compiles the reference's own learnBestFeature OpenCL kernel
 * (src/padenti/kernels/learn_best_feature.cl:22-111) as C, one work-item at a
 * time, so the oracle's split rule can be checked against the reference code on
 * the same histograms.  The kernel uses no local memory and no barriers, so a
 * sequential loop over work-items is an exact execution of its NDRange.
 * log2 on a float argument resolves to log2f through <tgmath.h>, as the OpenCL
 * overload does.  Test infrastructure only.
 */
#include <stddef.h>
#include <tgmath.h>

static size_t ref_gid;
#define __kernel
#define __global
#define get_global_id(dim) (ref_gid)

#include <padenti/kernels/learn_best_feature.cl>

void ref_learn_best_feature(unsigned int *histogram, unsigned int *perClassTotSamples,
                            unsigned int nFeatures, unsigned int nThresholds,
                            unsigned int nClasses, unsigned int perThreadFeatThrPairs,
                            unsigned int *bestFeatures, unsigned int *bestThresholds,
                            float *entropies, size_t nThreads) {
  for (ref_gid = 0; ref_gid < nThreads; ref_gid++)
    learnBestFeature(histogram, perClassTotSamples, nFeatures, nThresholds, nClasses,
                     perThreadFeatThrPairs, bestFeatures, bestThresholds, entropies);
}
