// The broadphase tree shared by the step's kernels: an implicit 32-ary
// bounding-volume tree over the proxies' fat AABBs, leaves in Morton order
// (built and refit in broadphase.cu). Level 0 holds the leaves, level l has
// ceil(count[l-1] / 32) nodes, node k of level l bounding children
// 32k..32k+31 of level l-1; all levels share DWorld::nodeBox, level l
// starting at offset[l].
#pragma once

#include "dworld.cuh"

#define WIDE 32
#define WIDE_MAX_LEVELS 6

// Level sizes of the implicit tree over n leaves: level 0 holds the leaves,
// level l has ceil(count[l-1] / 32) nodes; all levels share nodeBox, level l
// starting at offset[l]. top is the root's level (0 when n == 1).
struct WideLevels
{
	int count[WIDE_MAX_LEVELS + 1];
	int offset[WIDE_MAX_LEVELS + 1];
	int top;
};

__device__ __forceinline__ WideLevels wide_levels( int n )
{
	WideLevels L;
	L.count[0] = n;
	L.offset[0] = 0;
	int off = n, c = n, k = 0;
	while ( c > 1 && k < WIDE_MAX_LEVELS )
	{
		c = ( c + WIDE - 1 ) / WIDE;
		k += 1;
		L.count[k] = c;
		L.offset[k] = off;
		off += c;
	}
	L.top = k;
	return L;
}


// Thread-level walk: calls leaf(leafIndex) for every leaf whose box overlaps
// q. One (node, next child) cursor per level; bounded by the node count.
template <class F> __device__ __forceinline__ bool tree_query( const DWorld& w, int n, fbox q, F leaf )
{
	if ( n <= 0 )
		return true;
	const WideLevels L = wide_levels( n );
	if ( L.top == 0 )
	{
		if ( box_overlaps( q, box_from4( w.nodeBox[0] ) ) )
			leaf( 0 );
		return true;
	}
	int nodeAt[WIDE_MAX_LEVELS + 1];
	int next[WIDE_MAX_LEVELS + 1];
	int level = L.top;
	nodeAt[level] = 0;
	next[level] = 0;
	for ( int guard = 0; guard < 4 * n + 64; ++guard )
	{
		int node = nodeAt[level];
		int c = next[level];
		int nchild = min( WIDE, L.count[level - 1] - node * WIDE );
		if ( c >= nchild )
		{
			if ( level == L.top )
				return true;
			level += 1;
			continue;
		}
		next[level] = c + 1;
		int child = node * WIDE + c;
		if ( !box_overlaps( q, box_from4( w.nodeBox[L.offset[level - 1] + child] ) ) )
			continue;
		if ( level == 1 )
			leaf( child );
		else
		{
			level -= 1;
			nodeAt[level] = child;
			next[level] = 0;
		}
	}
	return false;
}
