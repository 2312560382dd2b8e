// Run-time compilation of user feature plugins with NVRTC (pd_plugin_compile):
// the counterpart of the reference compiling the user's feature.cl into its
// OpenCL program (cl_tree_trainer_impl.hpp:73-198, cl_classifier_impl.hpp:72-140).
// The user's computeFeature is compiled together with the library's kernel
// headers (embedded at build time) for this GPU; feat_t and img_t come from the
// context's configuration, as the reference generates feat_type.cl.
#include <nvrtc.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "pd_hist_grid.cuh"
#include "pd_rtc.cuh"

namespace pd {

namespace {

struct EmbeddedSource {
  const char *name, *text;
};
const EmbeddedSource kSources[] = {
#include "pd_rtc_sources.inc"
};

std::string unit_source(const pd_config &c, const std::string &user) {
  std::string s;
  switch (c.img_type) {
    case PD_IMG_U8: s += "typedef unsigned char img_t;\n"; break;
    case PD_IMG_U16: s += "typedef unsigned short img_t;\n"; break;
    case PD_IMG_I16: s += "typedef short img_t;\n"; break;
    case PD_IMG_I32: s += "typedef int img_t;\n"; break;
    default: s += "typedef float img_t;\n"; break;
  }
  s += c.feat_type == PD_FEAT_I16 ? "typedef short feat_t;\n" : "typedef int feat_t;\n";
  s += "#define PD_FEAT_DIM " + std::to_string(c.feat_dim) + "\n";
  s += "#define PD_CHANNELS " + std::to_string(c.n_channels) + "\n";
  s += "#include \"pd_train_kernels.cuh\"\n#include \"pd_predict_kernels.cuh\"\n#include \"pd_user_plugin.cuh\"\n";
  s += "#line 1 \"feature.cu\"\n";
  s += user;
  s += "\n#include \"pd_user_plugin_impl.cuh\"\n";
  return s;
}

// Compiles the unit for `arch` and returns the cubin and the lowered names of
// the kernels named by `exprs`.
int compile_unit(const pd_config &c, const std::string &user, const std::string &arch,
                 const std::vector<std::string> &exprs, std::string *cubin, std::vector<std::string> *lowered,
                 std::string *log) {
  const std::string src = unit_source(c, user);
  std::vector<const char *> hn, ht;
  for (const auto &e : kSources) {
    hn.push_back(e.name);
    ht.push_back(e.text);
  }
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "plugin_unit.cu", (int)hn.size(), ht.data(), hn.data());
  PD_CHECK(r == NVRTC_SUCCESS, PD_ERR_CUDA, "nvrtcCreateProgram: %s", nvrtcGetErrorString(r));
  for (const auto &e : exprs) nvrtcAddNameExpression(prog, e.c_str());
  const std::string a = "-arch=" + arch;
  const char *opts[] = {a.c_str(), "-std=c++20", "-default-device", "-diag-suppress=177,550"};
  r = nvrtcCompileProgram(prog, 4, opts);
  size_t ls = 0;
  nvrtcGetProgramLogSize(prog, &ls);
  std::string lg(ls, '\0');
  if (ls) nvrtcGetProgramLog(prog, &lg[0]);
  while (!lg.empty() && (lg.back() == '\0' || lg.back() == '\n')) lg.pop_back();
  if (log) *log = lg;
  if (r != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return set_error(PD_ERR_INVALID, "feature plugin does not compile: %s", lg.substr(0, 1500).c_str());
  }
  if (cubin) {
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin->resize(n);
    nvrtcGetCUBIN(prog, &(*cubin)[0]);
  }
  if (lowered) {
    lowered->clear();
    for (const auto &e : exprs) {
      const char *low = nullptr;
      nvrtcGetLoweredName(prog, e.c_str(), &low);
      lowered->push_back(low ? low : "");
    }
  }
  nvrtcDestroyProgram(&prog);
  return PD_OK;
}

int load_kernels(const std::string &cubin, const std::vector<std::string> &names, cudaLibrary_t *lib,
                 std::vector<cudaKernel_t> *ks) {
  PD_CUDA(cudaLibraryLoadData(lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  ks->clear();
  for (const auto &n : names) {
    cudaKernel_t k = nullptr;
    PD_CUDA(cudaLibraryGetKernel(&k, *lib, n.c_str()));
    ks->push_back(k);
  }
  return PD_OK;
}

std::string device_arch(int device) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return "sm_103a";
  return "sm_" + std::to_string(p.major) + std::to_string(p.minor) + (p.major >= 9 ? "a" : "");
}

}  // namespace

struct RtcPlugin {
  std::string source, arch;
  std::vector<cudaLibrary_t> libs;
  RtcKernels base;
  std::map<int, cudaKernel_t> hist;  // TP * 16 + SPI
};

int rtc_kernels(pd_ctx *ctx, const RtcKernels **out) {
  PD_CHECK(ctx->rtc, PD_ERR_STATE, "the user feature plugin is not compiled (pd_plugin_compile)");
  *out = &ctx->rtc->base;
  return PD_OK;
}

int rtc_hist_kernel(pd_ctx *ctx, uint32_t TP, int SPI, cudaKernel_t *out) {
  PD_CHECK(ctx->rtc, PD_ERR_STATE, "the user feature plugin is not compiled (pd_plugin_compile)");
  const int key = (int)TP * 16 + SPI;
  auto it = ctx->rtc->hist.find(key);
  if (it != ctx->rtc->hist.end()) {
    *out = it->second;
    return PD_OK;
  }
  const std::vector<std::string> exprs = {"pd::k_hist<pd::UserPlugin, " + std::to_string(TP) + ", " +
                                          std::to_string(SPI) + ">"};
  std::string cubin;
  std::vector<std::string> low;
  PD_TRY(compile_unit(ctx->cfg, ctx->rtc->source, ctx->rtc->arch, exprs, &cubin, &low, nullptr));
  cudaLibrary_t lib = nullptr;
  std::vector<cudaKernel_t> ks;
  PD_TRY(load_kernels(cubin, low, &lib, &ks));
  ctx->rtc->libs.push_back(lib);
  ctx->rtc->hist[key] = ks[0];
  *out = ks[0];
  return PD_OK;
}

int rtc_set_smem(pd_ctx *ctx, cudaKernel_t k, size_t smem, int carveout_pct) {
  PD_CUDA(cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem, ctx->device));
  if (carveout_pct >= 0)
    PD_CUDA(cudaKernelSetAttributeForDevice(k, cudaFuncAttributePreferredSharedMemoryCarveout, carveout_pct,
                                            ctx->device));
  return PD_OK;
}

int rtc_launch(pd_ctx *ctx, cudaKernel_t k, dim3 grid, dim3 block, size_t smem, void **args) {
  PD_CUDA(cudaLaunchKernel((const void *)k, grid, block, args, smem, ctx->stream));
  ctx->launches++;
  return PD_OK;
}

// The histogram launch of a user feature: the same work list, shared memory
// and launch shapes as the compiled-in kernel (pd_hist_grid_impl.cuh), with
// k_hist<UserPlugin, TP, SPI> compiled for the context's GPU.
int launch_hist_grid_rtc(pd_ctx *ctx, const HistGrid &g) {
  const int spi = (int)ctx->hist_spi;
  const int resident = spi <= 2 ? 3 : 2;
  cudaKernel_t uk = nullptr;
  PD_TRY(rtc_hist_kernel(ctx, g.TP, spi, &uk));
  // shared memory carve-out for the resident CTAs (dynamic + a static allowance + reserved)
  const size_t per_cta = g.smem + 4096 + 1024;
  const int pct = (int)std::min<size_t>(100, (resident * per_cta * 100 + 233471) / 233472);
  PD_TRY(rtc_set_smem(ctx, uk, g.smem, pct));
  if (g.queue) PD_CUDA(cudaMemsetAsync(g.queue, 0, 4, ctx->stream));
  if (g.ev_before) PD_CUDA(cudaEventRecord(g.ev_before, ctx->stream));
  for (uint64_t b = 0; b < g.n_items; b += 0x7fffffffull) {
    const uint64_t cnt = std::min<uint64_t>(g.n_items - b, 0x7fffffffull);
    DevSet ds = g.ds;
    const SampleRec *rec = g.rec;
    const WorkItem *items = g.items + b;
    uint32_t n = (uint32_t)cnt;
    unsigned *queue = g.queue;
    const void *cf = g.cand_feat, *ct = g.cand_thr;
    uint32_t *hist = g.hist;
    uint32_t F = g.F, T = g.T, K = g.K;
    FusedSplit fs = g.fs;
    void *args[] = {&ds, &rec, &items, &n, &queue, &cf, &ct, &hist, &F, &T, &K, &fs};
    const unsigned grid = g.queue ? (unsigned)std::min<uint64_t>(cnt, (uint64_t)ctx->n_sms * resident) : (unsigned)cnt;
    PD_TRY(rtc_launch(ctx, uk, dim3(grid), dim3(kHistThreads), g.smem, args));
    if (g.queue) break;
  }
  return PD_OK;
}

void rtc_release(pd_ctx *ctx) {
  if (!ctx->rtc) return;
  for (cudaLibrary_t l : ctx->rtc->libs) cudaLibraryUnload(l);
  delete ctx->rtc;
  ctx->rtc = nullptr;
}

}  // namespace pd

using namespace pd;

extern "C" int pd_plugin_check(const pd_config *cfg, const char *source, char *log, size_t log_size) {
  PD_CHECK(cfg && source, PD_ERR_INVALID, "null argument");
  PD_CHECK(cfg->plugin == PD_PLUGIN_USER, PD_ERR_INVALID, "the configuration's plugin is not PD_PLUGIN_USER");
  std::string lg;
  const int rc = compile_unit(*cfg, source, "sm_103a",
                              {"pd::k_reassign<pd::UserPlugin>", "pd::k_predict_leaf<pd::UserPlugin>",
                               "pd::k_node_map_step<pd::UserPlugin>", "pd::k_hist<pd::UserPlugin, 16, 8>"},
                              nullptr,
                              nullptr, &lg);
  if (log && log_size) {
    const size_t n = std::min(log_size - 1, lg.size());
    memcpy(log, lg.data(), n);
    log[n] = '\0';
  }
  return rc;
}

extern "C" int pd_plugin_compile(pd_ctx *ctx, const char *source) {
  PD_CHECK(ctx && source, PD_ERR_INVALID, "null argument");
  PD_CHECK(is_user_plugin(ctx), PD_ERR_INVALID, "the context was not created for PD_PLUGIN_USER");
  PD_CUDA(cudaSetDevice(ctx->device));
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  auto *p = new RtcPlugin();
  p->source = source;
  p->arch = device_arch(ctx->device);
  const std::vector<std::string> exprs = {
      "pd::k_reassign<pd::UserPlugin>", "pd::k_build_rec<pd::UserPlugin>", "pd::k_cand_order<pd::UserPlugin>",
      "pd::k_predict_posterior<pd::UserPlugin>", "pd::k_predict_leaf<pd::UserPlugin>",
      "pd::k_predict_batch<pd::UserPlugin>", "pd::k_forest_nodes<pd::UserPlugin>",
      "pd::k_node_map_step<pd::UserPlugin>"};
  std::string cubin;
  std::vector<std::string> low;
  int rc = compile_unit(ctx->cfg, p->source, p->arch, exprs, &cubin, &low, nullptr);
  cudaLibrary_t lib = nullptr;
  std::vector<cudaKernel_t> ks;
  if (rc == PD_OK) rc = load_kernels(cubin, low, &lib, &ks);
  int reads_tree = 0, rec_bytes = 0;
  // the form of the user's computeFeature and the size of its node records, as the compiler saw them
  for (auto [name, dst] : {std::pair<const char *, int *>{"pd_user_reads_tree", &reads_tree},
                           std::pair<const char *, int *>{"pd_node_rec_bytes", &rec_bytes}}) {
    if (rc != PD_OK) break;
    void *g = nullptr;
    size_t bytes = 0;
    cudaError_t e = cudaLibraryGetGlobal(&g, &bytes, lib, name);
    if (e == cudaSuccess && bytes == sizeof(int)) e = cudaMemcpy(dst, g, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess || bytes != sizeof(int))
      rc = set_error(PD_ERR_CUDA, "reading %s from the plugin module: %s", name, cudaGetErrorString(e));
  }
  if (rc != PD_OK) {
    if (lib) cudaLibraryUnload(lib);
    delete p;
    return rc;
  }
  p->libs.push_back(lib);
  p->base.reassign = ks[0];
  p->base.build_rec = ks[1];
  p->base.cand_order = ks[2];
  p->base.predict_posterior = ks[3];
  p->base.predict_leaf = ks[4];
  p->base.predict_batch = ks[5];
  p->base.forest_nodes = ks[6];
  p->base.node_map_step = ks[7];
  p->base.node_rec_bytes = rec_bytes;
  rtc_release(ctx);  // a previous plugin of this context
  ctx->rtc = p;
  ctx->tree_feature = reads_tree != 0;
  ctx->have_dataset = false;  // the sample records depend on the plugin: upload again
  return PD_OK;
}
