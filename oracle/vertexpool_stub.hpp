// TEST INFRASTRUCTURE (oracle only).
//
// No-op stand-in for the reference's GL vertex pool (source/vertexpool.hpp),
// which needs OpenGL. source/cellpool.h:268-333 (indexnode / updatenode) and
// :339-356 (map::init) name these members; the oracle never calls them, they
// only have to compile.
#pragma once

#include <cstddef>
#include <vector>

struct Vertex {
  Vertex(glm::vec3, glm::vec3, glm::vec3, glm::vec3) {}
};

template <typename T>
struct Vertexpool {
  std::vector<unsigned int> indices;
  unsigned int* section(int, int, glm::vec3, std::size_t) { return nullptr; }
  void resize(unsigned int*, std::size_t) {}
  void index() {}
  void update() {}
  void fill(unsigned int*, int, glm::vec3, glm::vec3, glm::vec3, glm::vec3) {}
  void reserve(int, int) {}
};
