// Structured box meshes and their node ordering, as the reference's mesh helpers produce them
// (symx/src/solver/mesh_generation.h, mesh_ordering.h): a box centred at the origin cut into
// Tet4 (6 per cell), Tet10 (the same split with mid-edge nodes), Hex8 or Hex27 elements, nodes
// renumbered by reverse Cuthill-McKee and elements reordered by a breadth-first walk of the
// element adjacency, so that user code built on these meshes gets the same numbering, and
// `enumerate` to prepend element indices to a connectivity.  Vertices are std::array (the
// reference stores Eigen vectors; the potentials accept either).
#pragma once

#include <array>
#include <cstdint>
#include <type_traits>
#include <utility>
#include <vector>

#include "fem.h"

namespace symx {

template <typename FLOAT>
struct FEMMesh {
    FEM_Element element_type = FEM_Element::Tet4;
    std::vector<std::array<FLOAT, 3>> vertices;
    std::vector<int> connectivity;
    int connectivity_stride = -1;
    int n_elements = -1;
};

// Each element of a flat connectivity (stride nodes each) prefixed with its 0-based index.
std::vector<int> enumerate(const std::vector<int>& connectivity, int stride);

struct ReorderResult {
    std::vector<int> old_to_new;
    std::vector<int> new_to_old;
};

// Node adjacency of a connectivity: neighbours deduplicated, ordered by (degree, index).
std::vector<std::vector<int>> build_adjacency(const int* conn, int conn_stride, int n_elements, int num_nodes);

// Renumber the nodes of `conn` in place by reverse Cuthill-McKee (one pseudo-peripheral root
// per connected component), then, when asked, reorder the elements by a breadth-first walk of
// the element adjacency (reversed).  Returns the node permutation.
ReorderResult reorder_connectivity_RCM(int* conn, int conn_stride, int n_elements, int num_nodes,
                                       bool also_reorder_elements = true);

template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Tet4_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& elements_per_axis);
template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Tet10_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& elements_per_axis);
template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Hex8_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& elements_per_axis);
template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Hex27_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& elements_per_axis);
template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_mesh(const FEM_Element& elem, const std::array<FLOAT, 3>& size,
                                    const std::array<int32_t, 3>& elements_per_axis);

// The reference takes the box size as an Eigen 3-vector: any indexable 3-vector is accepted.
#define SYMX_MESH_VECTOR_OVERLOAD(NAME)                                                                          \
    template <typename V, typename FLOAT = std::decay_t<decltype(std::declval<const V&>()[0])>>                 \
    FEMMesh<FLOAT> NAME(const V& size, const std::array<int32_t, 3>& elements_per_axis)                         \
    {                                                                                                             \
        return NAME<FLOAT>(std::array<FLOAT, 3>{size[0], size[1], size[2]}, elements_per_axis);                  \
    }
SYMX_MESH_VECTOR_OVERLOAD(generate_cuboid_Tet4_mesh)
SYMX_MESH_VECTOR_OVERLOAD(generate_cuboid_Tet10_mesh)
SYMX_MESH_VECTOR_OVERLOAD(generate_cuboid_Hex8_mesh)
SYMX_MESH_VECTOR_OVERLOAD(generate_cuboid_Hex27_mesh)
#undef SYMX_MESH_VECTOR_OVERLOAD
template <typename V, typename FLOAT = std::decay_t<decltype(std::declval<const V&>()[0])>>
FEMMesh<FLOAT> generate_cuboid_mesh(const FEM_Element& elem, const V& size, const std::array<int32_t, 3>& elements_per_axis)
{
    return generate_cuboid_mesh<FLOAT>(elem, std::array<FLOAT, 3>{size[0], size[1], size[2]}, elements_per_axis);
}

}  // namespace symx
