// Edge order of the reference's mesh (TEST INFRASTRUCTURE ONLY).
//
// load_mesh keys its edges by Cantor's pairing of the sorted corner ids in
// an std::unordered_map<int, Edge> and copies them into Mesh::edges in the
// map's iteration order (include/load_mesh.hpp:17-22, 34-62, 146-206).  That
// order belongs to the standard library's container, so it is reproduced by
// inserting the same int keys, in the same sequence, into the same container.
// Only the dot product's edge sum (include/openmp_impl/dot.hpp:30-50)
// depends on it.
#include <unordered_map>

extern "C" void or_stl_edge_order(int n_edges, const int* keys, int* order)
{
    std::unordered_map<int, int> map;
    for (int k = 0; k < n_edges; ++k) map[keys[k]] = k;
    int pos = 0;
    for (const auto& kv : map) order[pos++] = kv.second;
}
