// Host copy of the broadphase trees: the creation-path half of Box2D
// v3.1.1's dynamic tree (packages/forge2d/third_party/box2d/src/
// dynamic_tree.c). The tree's topology fixes the order in which the world
// step creates contacts, so the GPU world keeps the reference's trees
// exactly: the host inserts and removes proxies (create, move, destroy; the
// SAH sibling search with rotations, :187-825) on this copy and uploads it;
// the device enlarges proxies and rebuilds the enlarged part every step
// (proxytree.cu). Node arrays use the device layout so that they move as
// whole arrays.
#pragma once

#include "dworld.cuh"

#include <vector>

struct HTree
{
	// per node id; a free node's `parent` is the next node of the free list
	std::vector<int> child1, child2, parent, height, flags, shape, leaves;
	std::vector<float4> box; // lower.x lower.y upper.x upper.y
	std::vector<unsigned long long> cat;
	int cap = 0, count = 0, freeList = -1, root = -1, proxyCount = 0;

	HTree();
	int create_proxy( float4 aabb, unsigned long long category, int shapeId );
	void destroy_proxy( int proxyId );
	void move_proxy( int proxyId, float4 aabb );
	void set_category( int proxyId, unsigned long long category );
	// leaf shapes in the order a depth-first query visits them
	void visit_order( std::vector<int>& shapes ) const;

  private:
	int alloc_node();
	void free_node( int id );
	void refresh( int id, bool keepEnlarged );
	int best_sibling( float4 d ) const;
	void swap_in( int a, int top, int low, int g, int keep, int topSlot, int lowSlot, float4 lowBox );
	void rotate( int a );
	void insert_leaf( int leaf, bool shouldRotate );
	void remove_leaf( int leaf );
};
