// Tree<FeatType, FeatDim, nClasses> -- a complete binary heap of 2^depth - 1
// nodes kept as separate arrays, the layout of the reference tree
// (tree.hpp:72-173): leftChild is -2 for an absent node, -1 for a leaf and
// 2i+1 for a split node; features [node][FeatDim]; thresholds [node];
// posteriors [node][nClasses].  save()/load() read and write the reference's XML
// file (tree_impl.hpp:103-234: Boost.PropertyTree without indentation, absent
// nodes omitted, floats with six significant digits).
#ifndef PADENTI_GB300_TREE_HPP
#define PADENTI_GB300_TREE_HPP

#include <algorithm>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

template <typename FeatType, unsigned int FeatDim>
struct TreeNode {
  int *m_leftChild;
  FeatType *m_feature;
  FeatType *m_threshold;
  float *m_posterior;
};

template <typename FeatType, unsigned int FeatDim, unsigned int nClasses>
class Tree {
  unsigned int m_id = 0;
  unsigned int m_depth = 0;
  std::vector<int> m_leftChildren;
  std::vector<FeatType> m_features;
  std::vector<FeatType> m_thresholds;
  std::vector<float> m_posteriors;
  mutable TreeNode<FeatType, FeatDim> m_node{};

  void init() {
    const size_t n = m_depth ? ((size_t)1 << m_depth) - 1 : 0;
    m_leftChildren.assign(n, -2);
    m_features.assign(n * FeatDim, (FeatType)0);
    m_thresholds.assign(n, (FeatType)0);
    m_posteriors.assign(n * nClasses, 0.0f);
  }
  static std::string tag(const std::string &xml, const std::string &name, size_t from, size_t to) {
    const std::string open = "<" + name + ">", close = "</" + name + ">";
    const size_t b = xml.find(open, from);
    if (b == std::string::npos || b >= to) return std::string();
    const size_t e = xml.find(close, b);
    if (e == std::string::npos || e > to) return std::string();
    return xml.substr(b + open.size(), e - b - open.size());
  }

 public:
  Tree() = default;
  Tree(unsigned int id, unsigned int depth) : m_id(id), m_depth(depth) { init(); }
  unsigned int getID() const { return m_id; }
  unsigned int getDepth() const { return m_depth; }
  size_t getNNodes() const { return m_leftChildren.size(); }
  const TreeNode<FeatType, FeatDim> &getNode(unsigned int idx) const {
    auto *self = const_cast<Tree *>(this);
    m_node.m_leftChild = &self->m_leftChildren[idx];
    m_node.m_feature = &self->m_features[(size_t)idx * FeatDim];
    m_node.m_threshold = &self->m_thresholds[idx];
    m_node.m_posterior = &self->m_posteriors[(size_t)idx * nClasses];
    return m_node;
  }
  int *getLeftChildren() const { return const_cast<int *>(m_leftChildren.data()); }
  FeatType *getFeatures() const { return const_cast<FeatType *>(m_features.data()); }
  FeatType *getThresholds() const { return const_cast<FeatType *>(m_thresholds.data()); }
  float *getPosteriors() const { return const_cast<float *>(m_posteriors.data()); }

  std::string toXML(int idx = -1) const {
    std::ostringstream o;
    const unsigned int tid = idx == -1 ? m_id : (unsigned int)idx;
    o << "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n<Trees><TreeNumber>1</TreeNumber><MaxDepth>" << m_depth
      << "</MaxDepth><Tree" << tid << ">";
    for (size_t i = 0; i < m_leftChildren.size(); i++) {
      const int c = m_leftChildren[i];
      if (c == -2) continue;
      o << "<Node" << i << "><LeftChild>" << c << "</LeftChild>";
      if (c != -1) {
        o << "<SplitParameters>";
        for (unsigned int f = 0; f < FeatDim; f++) o << +m_features[i * FeatDim + f] << " ";
        o << +m_thresholds[i] << "</SplitParameters>";
      }
      o << "<Histogram>";
      for (unsigned int l = 0; l < nClasses; l++) o << (l ? " " : "") << m_posteriors[i * nClasses + l];
      o << "</Histogram></Node" << i << ">";
    }
    o << "</Tree" << tid << "></Trees>";
    return o.str();
  }
  void save(const std::string &path, int idx = -1) const {
    std::ofstream f(path);
    if (!f) throw std::runtime_error("cannot write " + path);
    f << toXML(idx);
  }
  void load(const std::string &path, int idx = -1) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot read " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string xml = ss.str();
    if (idx != -1) m_id = (unsigned int)idx;
    const std::string md = tag(xml, "MaxDepth", 0, xml.size());
    if (md.empty()) throw std::runtime_error(path + ": no MaxDepth");
    m_depth = (unsigned int)std::atoi(md.c_str());
    init();
    const std::string topen = "<Tree" + std::to_string(m_id) + ">";
    const size_t tb = xml.find(topen);
    if (tb == std::string::npos) return;
    const size_t te = xml.find("</Tree" + std::to_string(m_id) + ">", tb);
    // one pass over the <NodeI>...</NodeI> elements of this tree
    for (size_t pos = xml.find("<Node", tb); pos != std::string::npos && pos < te; pos = xml.find("<Node", pos)) {
      const size_t gt = xml.find('>', pos);
      const size_t i = (size_t)std::strtoull(xml.c_str() + pos + 5, nullptr, 10);
      const std::string close = "</Node" + std::to_string(i) + ">";
      const size_t end = xml.find(close, gt);
      if (gt == std::string::npos || end == std::string::npos || i >= m_leftChildren.size())
        throw std::runtime_error(path + ": malformed node element");
      const std::string body = xml.substr(gt + 1, end - gt - 1);
      pos = end + close.size();
      const int c = std::atoi(tag(body, "LeftChild", 0, body.size()).c_str());
      m_leftChildren[i] = c;
      std::istringstream hs(tag(body, "Histogram", 0, body.size()));
      for (unsigned int l = 0; l < nClasses; l++) hs >> m_posteriors[i * nClasses + l];
      if (c >= 0) {
        std::istringstream ps(tag(body, "SplitParameters", 0, body.size()));
        long v = 0;
        for (unsigned int f = 0; f < FeatDim; f++) {
          ps >> v;
          m_features[i * FeatDim + f] = (FeatType)v;
        }
        ps >> v;
        m_thresholds[i] = (FeatType)v;
      }
    }
  }
};

#endif
