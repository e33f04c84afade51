// Host check of the edge/face numbering of xg_mesh_create
// (ngsxfem_gb300/csrc/xg_topology.h) on meshes whose vertex numbers exceed
// 2^21: a structured Kuhn tetrahedral mesh whose vertices are renumbered by a
// random injective map into [0, 2^24).  The numbering must equal the rank of
// each sorted vertex tuple among the distinct tuples (std::set order), and the
// counts must match the Euler relation of the mesh.  Exit status 1 on a
// mismatch.
#include <cstdio>
#include <random>
#include <set>
#include <unordered_set>

#include "xg_topology.h"

using namespace xg;

int main() {
  const int n = 12, nv1 = n + 1, nv = nv1 * nv1 * nv1, ne = 6 * n * n * n;
  std::mt19937_64 g(20261203);
  std::uniform_int_distribution<int32_t> U(0, (1 << 24) - 1);
  std::vector<int32_t> perm(nv);
  std::unordered_set<int32_t> used;
  for (int v = 0; v < nv; v++) {
    int32_t x;
    do x = U(g); while (!used.insert(x).second);
    perm[v] = x;
  }
  auto vid = [&](int i, int j, int k) { return perm[(k * nv1 + j) * nv1 + i]; };
  static const int path[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  std::vector<int32_t> elv;
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++)
        for (int p = 0; p < 6; p++) {
          int c[3] = {i, j, k};
          elv.push_back(vid(c[0], c[1], c[2]));
          for (int s = 0; s < 3; s++) {
            c[path[p][s]]++;
            elv.push_back(vid(c[0], c[1], c[2]));
          }
        }
  std::vector<int32_t> el_edges, el_faces;
  const int64_t nedges = number_edges(3, ne, elv.data(), el_edges);
  const int64_t nfaces = number_faces(ne, elv.data(), el_faces);

  std::set<std::array<int32_t, 3>> fs;
  std::set<std::pair<int32_t, int32_t>> es;
  for (int e = 0; e < ne; e++) {
    for (int j = 0; j < 4; j++) {
      std::array<int32_t, 3> f;
      for (int q = 0; q < 3; q++) f[q] = elv[(size_t)e * 4 + TET_FACES[j][q]];
      std::sort(f.begin(), f.end());
      fs.insert(f);
    }
    for (int j = 0; j < 6; j++) {
      int a = elv[(size_t)e * 4 + TET_EDGES[j][0]], b = elv[(size_t)e * 4 + TET_EDGES[j][1]];
      es.insert({std::min(a, b), std::max(a, b)});
    }
  }
  int bad = 0;
  // Euler: V - E + F - T = 1 for a contractible tetrahedral mesh
  if ((int64_t)nv - nedges + nfaces - ne != 1) {
    printf("Euler relation fails: V=%d E=%lld F=%lld T=%d\n", nv, (long long)nedges, (long long)nfaces, ne);
    bad++;
  }
  if ((size_t)nfaces != fs.size() || (size_t)nedges != es.size()) {
    printf("counts: faces %lld vs %zu, edges %lld vs %zu\n", (long long)nfaces, fs.size(), (long long)nedges, es.size());
    bad++;
  }
  std::vector<std::array<int32_t, 3>> fv(fs.begin(), fs.end());
  std::vector<std::pair<int32_t, int32_t>> ev(es.begin(), es.end());
  for (int e = 0; e < ne && bad < 10; e++) {
    for (int j = 0; j < 4; j++) {
      std::array<int32_t, 3> f;
      for (int q = 0; q < 3; q++) f[q] = elv[(size_t)e * 4 + TET_FACES[j][q]];
      std::sort(f.begin(), f.end());
      const int32_t id = el_faces[(size_t)e * 4 + j];
      if (id < 0 || (size_t)id >= fv.size() || fv[id] != f) {
        printf("face (%d,%d,%d) of element %d numbered %d\n", f[0], f[1], f[2], e, id);
        bad++;
      }
    }
    for (int j = 0; j < 6; j++) {
      int a = elv[(size_t)e * 4 + TET_EDGES[j][0]], b = elv[(size_t)e * 4 + TET_EDGES[j][1]];
      const int32_t id = el_edges[(size_t)e * 6 + j];
      if (id < 0 || (size_t)id >= ev.size() || ev[id] != std::make_pair(std::min(a, b), std::max(a, b))) {
        printf("edge (%d,%d) of element %d numbered %d\n", a, b, e, id);
        bad++;
      }
    }
  }
  printf("%d vertices numbered up to 2^24, %lld edges, %lld faces: %s\n", nv, (long long)nedges,
         (long long)nfaces, bad ? "MISMATCH" : "ok");
  return bad ? 1 : 0;
}
