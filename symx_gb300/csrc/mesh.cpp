#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <queue>
#include <stdexcept>

namespace symx {

std::vector<int> enumerate(const std::vector<int>& connectivity, int stride)
{
    if (stride <= 0) throw std::invalid_argument("symx: enumerate needs a positive stride");
    const size_t n = connectivity.size() / (size_t)stride;
    std::vector<int> out;
    out.reserve(n * (stride + 1));
    for (size_t e = 0; e < n; ++e) {
        out.push_back((int)e);
        out.insert(out.end(), connectivity.begin() + e * stride, connectivity.begin() + (e + 1) * stride);
    }
    return out;
}

std::vector<std::vector<int>> build_adjacency(const int* conn, int conn_stride, int n_elements, int num_nodes)
{
    std::vector<std::vector<int>> adj(num_nodes);
    for (int e = 0; e < n_elements; ++e) {
        const int* c = conn + (size_t)e * conn_stride;
        for (int i = 0; i < conn_stride; ++i)
            for (int j = i + 1; j < conn_stride; ++j)
                if (c[i] != c[j]) {
                    adj[c[i]].push_back(c[j]);
                    adj[c[j]].push_back(c[i]);
                }
    }
    std::vector<int> deg(num_nodes);
    for (int v = 0; v < num_nodes; ++v) {
        std::sort(adj[v].begin(), adj[v].end());
        adj[v].erase(std::unique(adj[v].begin(), adj[v].end()), adj[v].end());
        deg[v] = (int)adj[v].size();
    }
    for (auto& nb : adj)
        std::sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; });
    return adj;
}

namespace {

// Breadth-first order from `root` over the nodes with allowed[v] set (all when null), marking
// them in `seen`.
std::vector<int> bfs_order(const std::vector<std::vector<int>>& adj, int root, std::vector<char>& seen,
                           const std::vector<char>* allowed)
{
    std::vector<int> order;
    std::queue<int> q;
    q.push(root);
    seen[root] = 1;
    while (!q.empty()) {
        const int u = q.front();
        q.pop();
        order.push_back(u);
        for (int v : adj[u])
            if (!seen[v] && (!allowed || (*allowed)[v])) {
                seen[v] = 1;
                q.push(v);
            }
    }
    return order;
}

// Last node reached by a breadth-first search from `src`.
int bfs_last(const std::vector<std::vector<int>>& adj, int src)
{
    std::vector<char> seen(adj.size(), 0);
    return bfs_order(adj, src, seen, nullptr).back();
}

// Reverse Cuthill-McKee: per connected component (in order of its smallest node index), the
// root is found by two breadth-first sweeps from the component's first node of least degree,
// the breadth-first order from the root (neighbours by degree, then index) is reversed, and
// the components' orders are concatenated.  Returns new index of each old node.
std::vector<int> rcm_old_to_new(const std::vector<std::vector<int>>& adj)
{
    const int n = (int)adj.size();
    std::vector<char> done(n, 0), in_comp(n, 0);
    std::vector<int> order;
    order.reserve(n);
    for (int first = 0; first < n; ++first) {
        if (done[first]) continue;
        std::vector<char> seen(n, 0);
        const std::vector<int> comp = bfs_order(adj, first, seen, nullptr);
        int start = comp[0];
        for (int u : comp)
            if (adj[u].size() < adj[start].size()) start = u;
        const int root = bfs_last(adj, bfs_last(adj, start));
        for (int u : comp) in_comp[u] = 1;
        std::vector<int> level = bfs_order(adj, root, done, &in_comp);
        for (int u : comp) in_comp[u] = 0;
        order.insert(order.end(), level.rbegin(), level.rend());
    }
    std::vector<int> old_to_new(n);
    for (int i = 0; i < n; ++i) old_to_new[order[i]] = i;
    return old_to_new;
}

// Element order: breadth-first walks of the element adjacency (elements sharing a node),
// each from the unvisited element of least (degree, key) with key = (smallest node << 16) ^
// mean node index, visiting neighbours by (shared nodes desc, degree, index).
std::vector<int> element_bfs_order(const int* conn, int stride, int n_elements, int num_nodes)
{
    std::vector<std::vector<int>> incident(num_nodes);
    for (int e = 0; e < n_elements; ++e)
        for (int i = 0; i < stride; ++i) incident[conn[(size_t)e * stride + i]].push_back(e);
    std::vector<std::vector<int>> adj(n_elements);
    for (const auto& el : incident)
        for (size_t i = 0; i < el.size(); ++i)
            for (size_t j = i + 1; j < el.size(); ++j) {
                adj[el[i]].push_back(el[j]);
                adj[el[j]].push_back(el[i]);
            }
    std::vector<int> deg(n_elements), key(n_elements);
    for (int e = 0; e < n_elements; ++e) {
        std::sort(adj[e].begin(), adj[e].end());
        adj[e].erase(std::unique(adj[e].begin(), adj[e].end()), adj[e].end());
        deg[e] = (int)adj[e].size();
        const int* c = conn + (size_t)e * stride;
        int mn = c[0];
        long long sum = 0;
        for (int i = 0; i < stride; ++i) {
            mn = std::min(mn, c[i]);
            sum += c[i];
        }
        key[e] = (mn << 16) ^ (int)(sum / stride);
    }
    auto shared = [&](int a, int b) {
        int s = 0;
        const int* ca = conn + (size_t)a * stride;
        const int* cb = conn + (size_t)b * stride;
        for (int i = 0; i < stride; ++i)
            for (int j = 0; j < stride; ++j) s += ca[i] == cb[j];
        return s;
    };
    std::vector<char> seen(n_elements, 0);
    std::vector<int> order;
    order.reserve(n_elements);
    for (;;) {
        int seed = -1;
        for (int e = 0; e < n_elements; ++e)
            if (!seen[e] && (seed < 0 || deg[e] < deg[seed] || (deg[e] == deg[seed] && key[e] < key[seed]))) seed = e;
        if (seed < 0) break;
        std::queue<int> q;
        q.push(seed);
        seen[seed] = 1;
        while (!q.empty()) {
            const int u = q.front();
            q.pop();
            order.push_back(u);
            std::vector<int> nb = adj[u];
            std::vector<int> sh(nb.size());
            for (size_t k = 0; k < nb.size(); ++k) sh[k] = shared(u, nb[k]);
            std::vector<size_t> idx(nb.size());
            for (size_t k = 0; k < idx.size(); ++k) idx[k] = k;
            std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
                if (sh[a] != sh[b]) return sh[a] > sh[b];
                if (deg[nb[a]] != deg[nb[b]]) return deg[nb[a]] < deg[nb[b]];
                return nb[a] < nb[b];
            });
            for (size_t k : idx)
                if (!seen[nb[k]]) {
                    seen[nb[k]] = 1;
                    q.push(nb[k]);
                }
        }
    }
    return order;
}

template <typename FLOAT>
void renumber(FEMMesh<FLOAT>& mesh)
{
    mesh.n_elements = (int)(mesh.connectivity.size() / mesh.connectivity_stride);
    const ReorderResult r = reorder_connectivity_RCM(mesh.connectivity.data(), mesh.connectivity_stride,
                                                     mesh.n_elements, (int)mesh.vertices.size());
    std::vector<std::array<FLOAT, 3>> v(mesh.vertices.size());
    for (size_t i = 0; i < v.size(); ++i) v[r.old_to_new[i]] = mesh.vertices[i];
    mesh.vertices.swap(v);
}

// Grid of (sub n0 + 1) x (sub n1 + 1) x (sub n2 + 1) points spanning `size`, centred at the
// origin.  Each coordinate is one fused multiply-add, min + i * spacing, on every host (the
// reference's release build fuses it in most components; any difference is one rounding).
template <typename FLOAT>
void grid_vertices(FEMMesh<FLOAT>& mesh, const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& cells, int sub)
{
    std::array<FLOAT, 3> lo, d;
    for (int k = 0; k < 3; ++k) {
        lo[k] = FLOAT(-0.5) * size[k];
        d[k] = size[k] / (FLOAT)cells[k] / (FLOAT)sub;
    }
    for (int i = 0; i <= sub * cells[0]; ++i)
        for (int j = 0; j <= sub * cells[1]; ++j)
            for (int k = 0; k <= sub * cells[2]; ++k)
                mesh.vertices.push_back({std::fma((FLOAT)i, d[0], lo[0]), std::fma((FLOAT)j, d[1], lo[1]),
                                         std::fma((FLOAT)k, d[2], lo[2])});
}

void check_cells(const std::array<int32_t, 3>& cells)
{
    for (int k = 0; k < 3; ++k)
        if (cells[k] <= 0) throw std::invalid_argument("symx: elements per axis must be positive");
}

// Corners of cell (i, j, k) in the split's order, on a grid of stride `s` per cell.
struct Cell {
    int n1, n2, s, i, j, k;
    int at(int a, int b, int c) const { return (a * (n1 + 1) + b) * (n2 + 1) + c; }
    int corner(int q) const
    {
        static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        return at(i + s * off[q][0], j + s * off[q][1], k + s * off[q][2]);
    }
};

// The six tetrahedra of a cell around its diagonal 0-6 (corner indices), as the reference
// splits it (mesh_generation.cpp:76-83; its comment says 5, the code emits 6).
const int kTets[6][4] = {{0, 1, 6, 5}, {0, 1, 2, 6}, {0, 2, 3, 6}, {0, 5, 6, 4}, {0, 6, 3, 7}, {0, 6, 7, 4}};

}  // namespace

ReorderResult reorder_connectivity_RCM(int* conn, int conn_stride, int n_elements, int num_nodes, bool also_reorder_elements)
{
    const std::vector<std::vector<int>> adj = build_adjacency(conn, conn_stride, n_elements, num_nodes);
    ReorderResult r;
    r.old_to_new = rcm_old_to_new(adj);
    r.new_to_old.resize(num_nodes);
    for (int i = 0; i < num_nodes; ++i) r.new_to_old[r.old_to_new[i]] = i;
    for (size_t i = 0; i < (size_t)n_elements * conn_stride; ++i) conn[i] = r.old_to_new[conn[i]];
    if (also_reorder_elements) {
        const std::vector<int> order = element_bfs_order(conn, conn_stride, n_elements, num_nodes);
        std::vector<int> out((size_t)n_elements * conn_stride);
        for (int e = 0; e < n_elements; ++e)  // the walk's order, reversed
            std::copy(conn + (size_t)order[n_elements - 1 - e] * conn_stride,
                      conn + (size_t)(order[n_elements - 1 - e] + 1) * conn_stride, out.begin() + (size_t)e * conn_stride);
        std::copy(out.begin(), out.end(), conn);
    }
    return r;
}

template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Tet4_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& cells)
{
    check_cells(cells);
    FEMMesh<FLOAT> mesh;
    mesh.element_type = FEM_Element::Tet4;
    mesh.connectivity_stride = 4;
    grid_vertices(mesh, size, cells, 1);
    for (int i = 0; i < cells[0]; ++i)
        for (int j = 0; j < cells[1]; ++j)
            for (int k = 0; k < cells[2]; ++k) {
                const Cell c{cells[1], cells[2], 1, i, j, k};
                for (const auto& t : kTets)
                    for (int a = 0; a < 4; ++a) mesh.connectivity.push_back(c.corner(t[a]));
            }
    renumber(mesh);
    return mesh;
}

template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Tet10_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& cells)
{
    check_cells(cells);
    FEMMesh<FLOAT> mesh;
    mesh.element_type = FEM_Element::Tet10;
    mesh.connectivity_stride = 10;
    grid_vertices(mesh, size, cells, 2);  // every point of the doubled grid (the reference keeps the unused ones too)
    const int n1 = 2 * cells[1], n2 = 2 * cells[2];
    for (int i = 0; i < 2 * cells[0]; i += 2)
        for (int j = 0; j < n1; j += 2)
            for (int k = 0; k < n2; k += 2) {
                const Cell c{n1, n2, 2, i, j, k};
                auto mid = [&](int p, int q) {
                    static const int off[8][3] = {{0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0},
                                                  {0, 0, 2}, {2, 0, 2}, {2, 2, 2}, {0, 2, 2}};
                    return c.at(i + (off[p][0] + off[q][0]) / 2, j + (off[p][1] + off[q][1]) / 2,
                                k + (off[p][2] + off[q][2]) / 2);
                };
                for (const auto& t : kTets) {
                    for (int a = 0; a < 4; ++a) mesh.connectivity.push_back(c.corner(t[a]));
                    // mid-edge nodes (0,1), (1,2), (0,2), (0,3), (1,3), (2,3) of the tetrahedron
                    const int edges[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
                    for (const auto& ed : edges) mesh.connectivity.push_back(mid(t[ed[0]], t[ed[1]]));
                }
            }
    renumber(mesh);
    return mesh;
}

template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Hex8_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& cells)
{
    check_cells(cells);
    FEMMesh<FLOAT> mesh;
    mesh.element_type = FEM_Element::Hex8;
    mesh.connectivity_stride = 8;
    grid_vertices(mesh, size, cells, 1);
    for (int i = 0; i < cells[0]; ++i)
        for (int j = 0; j < cells[1]; ++j)
            for (int k = 0; k < cells[2]; ++k) {
                const Cell c{cells[1], cells[2], 1, i, j, k};
                for (int q = 0; q < 8; ++q) mesh.connectivity.push_back(c.corner(q));
            }
    renumber(mesh);
    return mesh;
}

template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_Hex27_mesh(const std::array<FLOAT, 3>& size, const std::array<int32_t, 3>& cells)
{
    check_cells(cells);
    FEMMesh<FLOAT> mesh;
    mesh.element_type = FEM_Element::Hex27;
    mesh.connectivity_stride = 27;
    grid_vertices(mesh, size, cells, 2);
    const int n1 = 2 * cells[1], n2 = 2 * cells[2];
    // node order of the reference's Hex27 (mesh_generation.cpp:253-295): corners (bottom, top),
    // mid-edges (bottom, top, vertical), face centres, cell centre; offsets in half cells
    static const int nodes[27][3] = {
        {0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2}, {0, 2, 2},
        {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {1, 0, 2}, {2, 1, 2}, {1, 2, 2}, {0, 1, 2},
        {0, 0, 1}, {2, 0, 1}, {2, 2, 1}, {0, 2, 1},
        {0, 1, 1}, {2, 1, 1}, {1, 2, 1}, {1, 0, 1}, {1, 1, 0}, {1, 1, 2},
        {1, 1, 1}};
    for (int i = 0; i < 2 * cells[0]; i += 2)
        for (int j = 0; j < n1; j += 2)
            for (int k = 0; k < n2; k += 2) {
                const Cell c{n1, n2, 2, i, j, k};
                for (const auto& o : nodes) mesh.connectivity.push_back(c.at(i + o[0], j + o[1], k + o[2]));
            }
    renumber(mesh);
    return mesh;
}

template <typename FLOAT>
FEMMesh<FLOAT> generate_cuboid_mesh(const FEM_Element& elem, const std::array<FLOAT, 3>& size,
                                    const std::array<int32_t, 3>& cells)
{
    switch (elem) {
        case FEM_Element::Tet4: return generate_cuboid_Tet4_mesh(size, cells);
        case FEM_Element::Tet10: return generate_cuboid_Tet10_mesh(size, cells);
        case FEM_Element::Hex8: return generate_cuboid_Hex8_mesh(size, cells);
        case FEM_Element::Hex27: return generate_cuboid_Hex27_mesh(size, cells);
    }
    throw std::invalid_argument("symx: generate_cuboid_mesh() got an unsupported element type");
}

#define SYMX_MESH_INSTANTIATE(F)                                                                                    \
    template FEMMesh<F> generate_cuboid_Tet4_mesh<F>(const std::array<F, 3>&, const std::array<int32_t, 3>&);       \
    template FEMMesh<F> generate_cuboid_Tet10_mesh<F>(const std::array<F, 3>&, const std::array<int32_t, 3>&);      \
    template FEMMesh<F> generate_cuboid_Hex8_mesh<F>(const std::array<F, 3>&, const std::array<int32_t, 3>&);       \
    template FEMMesh<F> generate_cuboid_Hex27_mesh<F>(const std::array<F, 3>&, const std::array<int32_t, 3>&);      \
    template FEMMesh<F> generate_cuboid_mesh<F>(const FEM_Element&, const std::array<F, 3>&, const std::array<int32_t, 3>&);
SYMX_MESH_INSTANTIATE(float)
SYMX_MESH_INSTANTIATE(double)
#undef SYMX_MESH_INSTANTIATE

}  // namespace symx
