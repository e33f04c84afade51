// Host-side numbering of the edges and faces of a simplex mesh (shared by
// xg_mesh_create and the native host check of the numbering).
//
// Edges are the unique (min, max) vertex pairs and faces the unique sorted
// vertex triples of all elements, numbered in lexicographic order of their
// vertex tuples, as NGSolve's MeshAccess numbers the edges/faces of the
// structured meshes that the reference's tests build.  Both keys keep full
// 32-bit vertex fields, so every vertex count that fits int32 numbers
// uniquely.
#pragma once
#include <algorithm>
#include <array>
#include <cstdint>
#include <vector>

namespace xg {

constexpr int TRI_EDGES[3][2] = {{0, 1}, {0, 2}, {1, 2}};
constexpr int TET_EDGES[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
constexpr int TET_FACES[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

// el_edges[e * nel + j] = number of local edge j of element e; returns the edge count
inline int64_t number_edges(int dim, int ne, const int32_t* elv, std::vector<int32_t>& el_edges) {
  const int nvl = dim + 1, nel = dim == 2 ? 3 : 6;
  std::vector<uint64_t> keys((size_t)ne * nel);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nel; j++) {
      int a = elv[(size_t)e * nvl + (dim == 2 ? TRI_EDGES[j][0] : TET_EDGES[j][0])];
      int b = elv[(size_t)e * nvl + (dim == 2 ? TRI_EDGES[j][1] : TET_EDGES[j][1])];
      if (a > b) std::swap(a, b);
      keys[(size_t)e * nel + j] = ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
    }
  std::vector<uint64_t> u(keys);
  std::sort(u.begin(), u.end());
  u.erase(std::unique(u.begin(), u.end()), u.end());
  el_edges.resize(keys.size());
  for (size_t i = 0; i < keys.size(); i++)
    el_edges[i] = (int32_t)(std::lower_bound(u.begin(), u.end(), keys[i]) - u.begin());
  return (int64_t)u.size();
}

// tetrahedra: el_faces[e * 4 + j] = number of local face j of element e;
// returns the face count
inline int64_t number_faces(int ne, const int32_t* elv, std::vector<int32_t>& el_faces) {
  using FaceKey = std::array<int32_t, 3>;
  std::vector<FaceKey> fk((size_t)ne * 4);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < 4; j++) {
      FaceKey v;
      for (int q = 0; q < 3; q++) v[q] = elv[(size_t)e * 4 + TET_FACES[j][q]];
      std::sort(v.begin(), v.end());
      fk[(size_t)e * 4 + j] = v;
    }
  std::vector<FaceKey> u(fk);
  std::sort(u.begin(), u.end());
  u.erase(std::unique(u.begin(), u.end()), u.end());
  el_faces.resize(fk.size());
  for (size_t i = 0; i < fk.size(); i++)
    el_faces[i] = (int32_t)(std::lower_bound(u.begin(), u.end(), fk[i]) - u.begin());
  return (int64_t)u.size();
}

}  // namespace xg
