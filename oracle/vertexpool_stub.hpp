// TEST INFRASTRUCTURE (oracle only).
//
// Stand-in for the reference's GL vertex pool (source/vertexpool.hpp), which
// needs OpenGL. source/cellpool.h:268-333 (indexnode / updatenode) and
// :339-356 (map::init) call these members. Nothing is drawn: `fill` records
// the four vectors updatenode writes for a vertex (position, normal, and the
// +x and +z edges, 12 floats) into `capture` when the harness points it at a
// buffer, so the oracle can compare the reference's own vertex data with the
// library's headless swe_world_vertices.
#pragma once

#include <cstddef>
#include <vector>

struct Vertex {
  Vertex(glm::vec3, glm::vec3, glm::vec3, glm::vec3) {}
};

template <typename T>
struct Vertexpool {
  std::vector<unsigned int> indices;
  float* capture = nullptr;  // 12 floats per vertex index, or nullptr
  unsigned int section_storage = 0;
  unsigned int* section(int, int, glm::vec3, std::size_t) { return &section_storage; }
  void resize(unsigned int*, std::size_t) {}
  void index() {}
  void update() {}
  void fill(unsigned int*, int i, glm::vec3 p, glm::vec3 n, glm::vec3 t, glm::vec3 b) {
    if (!capture) return;
    float* o = capture + 12 * (std::size_t)i;
    const glm::vec3 v[4] = {p, n, t, b};
    for (int k = 0; k < 4; k++) {
      o[3 * k + 0] = v[k].x;
      o[3 * k + 1] = v[k].y;
      o[3 * k + 2] = v[k].z;
    }
  }
  void reserve(int, int) {}
};
