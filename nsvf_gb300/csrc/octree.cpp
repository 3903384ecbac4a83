// Host-side sparse-voxel octree builder (the _ext.build_octree op).
//
// Reference: fairnr/clib/src/octree.cpp:13-136 (EasyOctree), which inserts
// every point with per-element at::Tensor operations (8.6 s for the
// 125,452-voxel c2 scene). This builder keeps the same tree and the same node
// numbering but stores nodes in a flat arena of plain structs: 32-bit child
// links instead of heap pointers, integer coordinates compared as FP32 like
// the reference's float centre tensor.
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/nsvf_gb300.h"

namespace {

struct Node {
  float c[3];     // centre (leaves hold their integer point)
  int32_t depth;  // -1 for leaves
  int32_t index;  // output row
  int32_t child[8];
};

// Builds the arena; returns false if a point lies outside the root cube.
int64_t build_arena(const float center[3], const int64_t *pts, int64_t npts, int depth,
                    std::vector<Node> &nodes, std::vector<int32_t> &bfs, int64_t &terminal) {
  nodes.clear();
  nodes.reserve((size_t)npts * 2 + 16);
  Node root;
  root.c[0] = center[0]; root.c[1] = center[1]; root.c[2] = center[2];
  root.depth = depth; root.index = -1;
  for (int i = 0; i < 8; ++i) root.child[i] = -1;
  nodes.push_back(root);
  for (int64_t k = 0; k < npts; ++k) {
    float p[3] = {(float)pts[k * 3 + 0], (float)pts[k * 3 + 1], (float)pts[k * 3 + 2]};
    int32_t cur = 0;
    for (;;) {
      // `point > center` as an FP32 comparison (octree.cpp:62-63)
      int dx = p[0] > nodes[cur].c[0], dy = p[1] > nodes[cur].c[1], dz = p[2] > nodes[cur].c[2];
      int ci = dx + 2 * dy + 4 * dz;
      if (nodes[cur].depth <= 0) {
        if (nodes[cur].depth < 0) return NSVF_ERR_INVALID;  // depth < 0 at the root
        // depth 0: the point becomes a leaf (a repeated point replaces the
        // earlier leaf, as in the reference)
        Node leaf;
        leaf.c[0] = p[0]; leaf.c[1] = p[1]; leaf.c[2] = p[2];
        leaf.depth = -1; leaf.index = (int32_t)k;
        for (int i = 0; i < 8; ++i) leaf.child[i] = -1;
        nodes.push_back(leaf);
        nodes[cur].child[ci] = (int32_t)(nodes.size() - 1);
        break;
      }
      if (nodes[cur].child[ci] < 0) {
        float len = (float)(1 << (nodes[cur].depth - 1));
        Node nn;
        nn.c[0] = nodes[cur].c[0] + (float)(2 * dx - 1) * len;
        nn.c[1] = nodes[cur].c[1] + (float)(2 * dy - 1) * len;
        nn.c[2] = nodes[cur].c[2] + (float)(2 * dz - 1) * len;
        nn.depth = nodes[cur].depth - 1; nn.index = -1;
        for (int i = 0; i < 8; ++i) nn.child[i] = -1;
        nodes.push_back(nn);
        nodes[cur].child[ci] = (int32_t)(nodes.size() - 1);
      }
      cur = nodes[cur].child[ci];
    }
  }
  // breadth-first order over the reachable nodes, children 0..7
  bfs.clear();
  bfs.reserve(nodes.size());
  bfs.push_back(0);
  terminal = 0;
  for (size_t h = 0; h < bfs.size(); ++h) {
    const Node &x = nodes[bfs[h]];
    if (x.depth == -1) terminal++;
    for (int i = 0; i < 8; ++i)
      if (x.child[i] >= 0) bfs.push_back(x.child[i]);
  }
  return (int64_t)bfs.size();
}

}  // namespace

extern "C" int64_t nsvf_build_octree(const float center[3], const int64_t *points,
                                     int64_t n_points, int depth, int32_t *centers,
                                     int32_t *children, int64_t capacity) {
  if (!center || (n_points > 0 && !points) || n_points < 0 || depth < 0 || depth > 29)
    return NSVF_ERR_INVALID;
  std::vector<Node> nodes;
  std::vector<int32_t> bfs;
  int64_t terminal = 0;
  int64_t total = build_arena(center, points, n_points, depth, nodes, bfs, terminal);
  if (total < 0) return total;
  if (!centers && !children) return total;  // size query
  if (!centers || !children) return NSVF_ERR_INVALID;
  if (capacity < total) return NSVF_ERR_CAPACITY;
  // Number the nodes: root = total-1, internal nodes count down in BFS order,
  // leaves keep their point index (octree.cpp:96-121).
  int64_t next = total - 1;
  nodes[0].index = (int32_t)next;
  for (size_t h = 0; h < bfs.size(); ++h) {
    Node &x = nodes[bfs[h]];
    for (int i = 0; i < 8; ++i) {
      int32_t c = x.child[i];
      if (c >= 0 && nodes[c].depth > -1) nodes[c].index = (int32_t)(--next);
    }
  }
  // A repeated point leaves a hole in the leaf numbering; the reference then
  // writes outside its tensors. Reject it.
  if (next != terminal) return NSVF_ERR_INVALID;
  // The surviving leaf ids must be exactly 0..terminal-1.
  for (size_t h = 0; h < bfs.size(); ++h) {
    const Node &x = nodes[bfs[h]];
    if (x.depth == -1 && (x.index < 0 || x.index >= terminal)) return NSVF_ERR_INVALID;
  }
  for (size_t h = 0; h < bfs.size(); ++h) {
    const Node &x = nodes[bfs[h]];
    int32_t *ch = children + (int64_t)x.index * 9;
    for (int i = 0; i < 8; ++i) ch[i] = x.child[i] >= 0 ? nodes[x.child[i]].index : -1;
    ch[8] = 1 << (x.depth + 1);
    for (int a = 0; a < 3; ++a) centers[(int64_t)x.index * 3 + a] = (int32_t)x.c[a];
  }
  return total;
}
