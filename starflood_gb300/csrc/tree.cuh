// tree.cuh -- device layout of the octree shared by the build, walk and export.
#pragma once

#include "internal.cuh"

constexpr uint32_t NODE_NONE = 0xFFFFFFFFu;

// Structure-of-arrays node records (16-byte vectors, one load per use):
//   geo    (mid x, mid y, mid z, w*w)       opening test, gravity.c:352-377
//   lo     (min x, min y, min z, max x)     self test, gravity.c:473-476
//   hi     (max y, max z, bodies, first child) as raw bits in .z/.w
//   com    (COM x, COM y, COM z, mass)      monopole, tree.c:302-310
//   parent, start (first sorted body)       export and monopoles
// Nodes are numbered: root 0; the children of the s-th split node in
// depth-first preorder are 1+8s .. 8+8s, in octant order.
// Each node is one 64-byte record of four float4 (geo, lo, hi, com), so the
// walk reads a node from a single cache line: node v's field X is
// nd.X[NODE_REC * v], the four pointers being offsets 0..3 into the records.
constexpr uint32_t NODE_REC = 4;
struct NodeArrays {
    float4* geo = nullptr;  // cell centre, w^2
    float4* lo = nullptr;   // min x, y, z, max x
    float4* hi = nullptr;   // max y, z, bodies, first child
    float4* com = nullptr;  // centre of mass, mass
    uint32_t* parent = nullptr;
    uint32_t* start = nullptr;
};

struct TreeWork {
    uint32_t n = 0, nodes_max = 0, split_cap = 0;
    uint64_t* keys = nullptr;   // sorted keys
    uint32_t* vals = nullptr;   // body index of each sorted slot
    SortWork sort;
    uint32_t* counters = nullptr;  // [0] bodies in cube [1] midplane bodies [2] moved midplane bodies [3] splits [4] max mass bits [5] gather's last-block ticket
    uint2* ties = nullptr;
    uint32_t* tie_pos = nullptr;   // moved midplane bodies: old slots ascending
    uint64_t* tie_key = nullptr;   // their new keys, ascending by (key, body)
    uint32_t* tie_body = nullptr;
    uint32_t* sbase = nullptr;
    uint32_t* split_start = nullptr;
    uint8_t* split_level = nullptr;
    uint32_t* split_node = nullptr;  // node id of each split node
    uint32_t* ordA = nullptr;        // EXACT monopoles: members in index order
    uint32_t* ordB = nullptr;
    NodeArrays nd;
    float4* sp = nullptr;       // sorted bodies (x, y, z, m)
    void* msum = nullptr;   // fixed-point (m x, m y, m z, m) per sorted slot (tree.cu fix4)
    void* cpre = nullptr;   // exclusive prefix of msum per 32 slots, then the total
    float4* walk_part = nullptr;  // split-walk partial sums (SPLIT x n)
};

size_t sf_walk_scratch_floats4(uint32_t n);

int sf_tree_build(sfgpu_sim* s);
int sf_walk_launch(sfgpu_sim* s);
