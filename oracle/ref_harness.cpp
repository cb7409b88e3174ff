/*
 * ORACLE — test infrastructure only.
 *
 * Headless C entry points around the reference's own CPU collision path,
 * compiled from the reference sources where they lie (see build_ref.sh):
 *   src/cpu/simpleBVH.cpp  SimpleBVH build / refit      (compiled unmodified)
 *   src/utils/utils.cpp    triangleIntersect, project6  (compiled unmodified)
 *
 * Two reference translation units are NOT compiled, because their object
 * construction binds an OpenGL context that does not exist here:
 *   src/utils/mesh.cpp       Mesh::Mesh creates GL vertex buffers (mesh.cpp:100-143)
 *   src/cpu/simpleCollide.cpp SimpleCollide::SimpleCollide creates GL buffers (:18-31)
 * In their place this file defines a headless Mesh constructor that only
 * stores vertices and indices (the fields SimpleBVH reads, simpleBVH.cpp:10-18,
 * 86-89), a no-op Transform (the CUDA helper a Mesh owns, transform.cu:8-16),
 * and a SimpleCollide whose detect() restates simpleCollide.cpp:47-161 line
 * for line over the reference-built SimpleBVH nodes, calling the reference's
 * own aabb_box_t::overlap and triangleIntersect.
 */
#include <iostream>
#include <mutex>
#include <sstream>
#include <stack>
#include <vector>

#include "cpu/simpleBVH.h"
#include "utils/utils.h"

Transform::Transform() : m_deviceVec4s(nullptr) {}
Transform::~Transform() {}

Mesh::Mesh(const std::vector<Vertex>& vertices,
           const std::vector<unsigned int>& indices,
           const std::vector<Texture>& textures)
    : m_verticesCount((unsigned int)vertices.size())
    , m_facesCount((unsigned int)(indices.size() / 3))
    , m_vertices(vertices)
    , m_indices(indices)
    , m_textures(textures)
{
}

Mesh::~Mesh() {}

/* SimpleBVH declares `friend class SimpleCollide` (include/cpu/simpleBVH.h:106). */
class SimpleCollide
{
public:
    struct Item
    {
        std::shared_ptr<simple_bvh_node_t> a, b;
        unsigned int ia, ib;
    };

    std::vector<std::shared_ptr<Mesh>> meshes;
    std::vector<std::shared_ptr<SimpleBVH>> bvhs;
    std::vector<int_tri_pair_node_t> hits;
    long long candidates = 0;

    void leafBoxes(unsigned int id, float* out6) const
    {
        std::stack<std::shared_ptr<simple_bvh_node_t>> st;
        st.push(bvhs[id]->m_root);
        while (!st.empty())
        {
            auto n = st.top();
            st.pop();
            if (n->m_triId != -1)
            {
                float* o = out6 + 6 * (size_t)n->m_triId;
                o[0] = n->m_aabb.m_minimum.x;
                o[1] = n->m_aabb.m_minimum.y;
                o[2] = n->m_aabb.m_minimum.z;
                o[3] = n->m_aabb.m_maximum.x;
                o[4] = n->m_aabb.m_maximum.y;
                o[5] = n->m_aabb.m_maximum.z;
                continue;
            }
            if (n->m_left)
                st.push(n->m_left);
            if (n->m_right)
                st.push(n->m_right);
        }
    }

    void detect(const std::vector<std::pair<unsigned int, unsigned int>>& pairs)
    {
        hits.clear();
        candidates = 0;
        std::stack<Item> st;
        for (const auto& pr : pairs)
        {
            st.push(Item{bvhs[pr.first]->m_root, bvhs[pr.second]->m_root, pr.first, pr.second});
            while (!st.empty())
            {
                const Item it = st.top();
                st.pop();
                if (!it.a->m_aabb.overlap(it.b->m_aabb))
                    continue;
                if (it.a->m_triId != -1 && it.b->m_triId != -1)
                {
                    candidates++;
                    const glm::uvec3 fa = bvhs[it.ia]->m_faces[it.a->m_triId];
                    const glm::uvec3 fb = bvhs[it.ib]->m_faces[it.b->m_triId];
                    const auto& pa = bvhs[it.ia]->m_positions;
                    const auto& pb = bvhs[it.ib]->m_positions;
                    if (triangleIntersect(pa[fa.x], pa[fa.y], pa[fa.z], pb[fb.x], pb[fb.y], pb[fb.z]))
                        hits.push_back(int_tri_pair_node_t{
                            {it.ia, it.ib}, {(unsigned int)it.a->m_triId, (unsigned int)it.b->m_triId}});
                    continue;
                }
                std::shared_ptr<simple_bvh_node_t> ca[2], cb[2];
                unsigned int na = 0, nb = 0;
                if (it.a->m_triId != -1)
                    ca[na++] = it.a;
                else
                {
                    ca[na++] = it.a->m_left;
                    if (it.a->m_right != nullptr)
                        ca[na++] = it.a->m_right;
                }
                if (it.b->m_triId != -1)
                    cb[nb++] = it.b;
                else
                {
                    cb[nb++] = it.b->m_left;
                    if (it.b->m_right != nullptr)
                        cb[nb++] = it.b->m_right;
                }
                for (unsigned int i = 0; i < na; i++)
                    for (unsigned int j = 0; j < nb; j++)
                        st.push(Item{ca[i], cb[j], it.ia, it.ib});
            }
        }
    }
};

namespace
{
/* std::cout is process-wide: the redirect is held under a lock, so that
 * scenes built on several threads at once (untimed set-up of the benches)
 * never restore each other's buffers. */
std::mutex g_cout_mu;
struct QuietCout
{
    std::lock_guard<std::mutex> lock;
    std::streambuf* saved;
    std::ostringstream sink;
    QuietCout() : lock(g_cout_mu), saved(std::cout.rdbuf(sink.rdbuf())) {}
    ~QuietCout() { std::cout.rdbuf(saved); }
};
} // namespace

extern "C" {

__attribute__((visibility("default"))) void* ref_scene_create()
{
    return new SimpleCollide();
}

__attribute__((visibility("default"))) void ref_scene_destroy(void* h)
{
    delete static_cast<SimpleCollide*>(h);
}

/* Mesh(vertices, indices) + SimpleBVH(mesh) + build(); returns the BVH id. */
__attribute__((visibility("default"))) int
ref_scene_add_mesh(void* h, const float* xyz, unsigned int nV, const unsigned int* tri, unsigned int nT)
{
    QuietCout quiet;
    auto* s = static_cast<SimpleCollide*>(h);
    std::vector<Vertex> verts(nV);
    for (unsigned int v = 0; v < nV; v++)
    {
        verts[v] = Vertex{};
        verts[v].m_position = glm::vec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
    }
    std::vector<unsigned int> idx(tri, tri + 3 * (size_t)nT);
    auto mesh = std::make_shared<Mesh>(verts, idx);
    auto bvh = std::make_shared<SimpleBVH>(mesh);
    bvh->build();
    s->meshes.push_back(mesh);
    s->bvhs.push_back(bvh);
    return (int)s->bvhs.size() - 1;
}

/* Move the mesh's vertices, then SimpleBVH::unRefit() + refit()
 * (the sequence at src/main.cpp:306-309). */
__attribute__((visibility("default"))) int ref_scene_set_positions(void* h, int id, const float* xyz)
{
    auto* s = static_cast<SimpleCollide*>(h);
    if (id < 0 || id >= (int)s->bvhs.size())
        return -1;
    auto& mesh = s->meshes[id];
    for (unsigned int v = 0; v < mesh->m_verticesCount; v++)
        mesh->m_vertices[v].m_position = glm::vec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
    s->bvhs[id]->unRefit();
    s->bvhs[id]->refit();
    return 0;
}

/* detect over the listed pairs (pairs == NULL: every i<j, as the reference). */
__attribute__((visibility("default"))) long long ref_scene_detect(
    void* h, const unsigned int* pairs, int n_pairs, unsigned int* out4, long long cap, long long* n_candidates)
{
    auto* s = static_cast<SimpleCollide*>(h);
    std::vector<std::pair<unsigned int, unsigned int>> pr;
    if (pairs)
        for (int p = 0; p < n_pairs; p++)
            pr.emplace_back(pairs[2 * p], pairs[2 * p + 1]);
    else
        for (unsigned int i = 0; i < s->bvhs.size(); i++)
            for (unsigned int j = i + 1; j < s->bvhs.size(); j++)
                pr.emplace_back(i, j);
    s->detect(pr);
    for (long long k = 0; k < (long long)s->hits.size() && k < cap; k++)
    {
        out4[4 * k + 0] = s->hits[k].m_bvhIndex[0];
        out4[4 * k + 1] = s->hits[k].m_bvhIndex[1];
        out4[4 * k + 2] = s->hits[k].m_triIndex[0];
        out4[4 * k + 3] = s->hits[k].m_triIndex[1];
    }
    if (n_candidates)
        *n_candidates = s->candidates;
    return (long long)s->hits.size();
}

/* The reference's triangleIntersect (src/utils/utils.cpp:97-169). */
__attribute__((visibility("default"))) int
ref_tri_intersect(const float* P1, const float* P2, const float* P3, const float* Q1, const float* Q2, const float* Q3)
{
    return triangleIntersect(glm::vec3(P1[0], P1[1], P1[2]),
                             glm::vec3(P2[0], P2[1], P2[2]),
                             glm::vec3(P3[0], P3[1], P3[2]),
                             glm::vec3(Q1[0], Q1[1], Q1[2]),
                             glm::vec3(Q2[0], Q2[1], Q2[2]),
                             glm::vec3(Q3[0], Q3[1], Q3[2]))
        ? 1
        : 0;
}

/* Leaf boxes of a reference SimpleBVH, written in original face order. */
__attribute__((visibility("default"))) int ref_scene_leaf_boxes(void* h, int id, float* out6)
{
    auto* s = static_cast<SimpleCollide*>(h);
    if (id < 0 || id >= (int)s->bvhs.size())
        return -1;
    s->leafBoxes((unsigned int)id, out6);
    return 0;
}

} // extern "C"
