// The reference's broadphase tree, restated. TEST INFRASTRUCTURE (oracle).
//
// Box2D v3.1.1 keeps one binary bounding-volume tree per body type
// (dynamic_tree.c). Its TOPOLOGY fixes three orders the world step exposes:
// the order new contacts are created in (broad_phase.c:311-474 walks each
// moved proxy's query in tree order), the order continuous collision visits
// static shapes (solver.c:444) and the order world queries and explosions
// report shapes (world.c:2071-2310, :2746). Proxy ids are node ids, so the
// node pool's LIFO free list fixes the proxy keys too. This file restates
// the tree operation by operation: node pool (dynamic_tree.c:80-185), SAH
// sibling choice and rotations on insert (:187-700), enlarge (:827-866),
// depth-first query (:1114-1170) and the partial rebuild with the median
// split the reference is compiled with (:1426-1989, B2_TREE_HEURISTIC 0).
#pragma once

#include "pmath.h"
#include <stdint.h>

// types.h:14 B2_DEFAULT_CATEGORY_BITS (the category of a fresh node)
#define P_DEFAULT_CATEGORY 1ull

enum
{
	RN_ALLOCATED = 1,
	RN_ENLARGED = 2,
	RN_LEAF = 4,
};

// 40 bytes, as the reference's node: children and the leaf's user data
// share their space
typedef struct RNode
{
	box2 aabb;
	uint64_t category;
	union
	{
		struct
		{
			int child1, child2; // internal nodes
		};
		int shape; // leaves: the shape id (the reference's user data)
	};
	int parent; // allocated: parent; free: next node of the free list
	uint16_t height; // 0 for leaves
	uint16_t flags;
} RNode;

typedef struct RTree
{
	RNode* nodes;
	int cap, count, freeList, root, proxyCount;
	// rebuild scratch (dynamic_tree.c:1872-1905)
	int* rbNode;
	v2* rbCenter;
	int rbCap;
} RTree;

void rt_init( RTree* t );
void rt_release_all( RTree* t );
int rt_create_proxy( RTree* t, box2 aabb, uint64_t category, int shape );
void rt_destroy_proxy( RTree* t, int proxyId );
void rt_move_proxy( RTree* t, int proxyId, box2 aabb );
void rt_enlarge_proxy( RTree* t, int proxyId, box2 aabb );
// rt_enlarge_proxy of `count` proxies at once (same result as the calls in
// any order)
void rt_enlarge_many( RTree* t, const int* proxies, const box2* boxes, int count );
void rt_set_category( RTree* t, int proxyId, uint64_t category );
int rt_rebuild( RTree* t, int fullBuild );

// depth-first query (dynamic_tree.c:1114): the visitor returns 0 to stop
typedef int ( *rt_visit_fn )( int proxyId, int shape, void* context );
void rt_query( const RTree* t, box2 aabb, uint64_t maskBits, rt_visit_fn fn, void* context );

// left-to-right rank of every leaf (child1 before child2), by node id;
// `rank` must hold t->cap entries. The query visits leaves in the reverse of
// this order.
void rt_leaf_ranks( const RTree* t, int* rank );
