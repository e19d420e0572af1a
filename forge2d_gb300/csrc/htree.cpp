// Host half of the broadphase trees (see htree.h). Each member cites the
// lines of packages/forge2d/third_party/box2d/src/dynamic_tree.c (v3.1.1)
// whose rule it follows; float expressions keep the reference's operand
// order because the chosen siblings and rotations decide the topology.
#include "htree.h"

#include <cfloat>

namespace
{
// b2AABB_Union with the reference's tie rule (the second operand wins ties)
inline float4 box_union( float4 a, float4 b )
{
	return make_float4( a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z > b.z ? a.z : b.z, a.w > b.w ? a.w : b.w );
}

// aabb.h:11-16 b2Perimeter
inline float perimeter( float4 a )
{
	float wx = a.z - a.x;
	float wy = a.w - a.y;
	return 2.0f * ( wx + wy );
}

inline float2 box_center( float4 a )
{
	return make_float2( 0.5f * ( a.x + a.z ), 0.5f * ( a.y + a.w ) );
}

inline int imax( int a, int b )
{
	return a > b ? a : b;
}
} // namespace

// :80-108: sixteen nodes, chained in ascending order on the free list
HTree::HTree()
{
	cap = 16;
	child1.assign( cap, -1 );
	child2.assign( cap, -1 );
	parent.resize( cap );
	height.assign( cap, 0 );
	flags.assign( cap, 0 );
	shape.assign( cap, -1 );
	leaves.assign( cap, 0 );
	box.assign( cap, make_float4( 0.0f, 0.0f, 0.0f, 0.0f ) );
	cat.assign( cap, 0ull );
	for ( int i = 0; i < cap; ++i )
		parent[i] = i + 1 < cap ? i + 1 : -1;
	freeList = 0;
}

// :122-158: pop the free list; an empty list grows the pool by half with
// the new nodes chained in ascending order
int HTree::alloc_node()
{
	if ( freeList == -1 )
	{
		int old = cap;
		cap = old + ( old >> 1 );
		child1.resize( cap, -1 );
		child2.resize( cap, -1 );
		parent.resize( cap, -1 );
		height.resize( cap, 0 );
		flags.resize( cap, 0 );
		shape.resize( cap, -1 );
		leaves.resize( cap, 0 );
		box.resize( cap, make_float4( 0.0f, 0.0f, 0.0f, 0.0f ) );
		cat.resize( cap, 0ull );
		for ( int i = count; i < cap; ++i )
			parent[i] = i + 1 < cap ? i + 1 : -1;
		freeList = count;
	}
	int id = freeList;
	freeList = parent[id];
	child1[id] = -1;
	child2[id] = -1;
	parent[id] = -1;
	height[id] = 0;
	flags[id] = PT_ALLOCATED;
	shape[id] = -1;
	leaves[id] = 0;
	box[id] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	cat[id] = 1ull; // B2_DEFAULT_CATEGORY_BITS
	count += 1;
	return id;
}

// :160-167
void HTree::free_node( int id )
{
	parent[id] = freeList;
	flags[id] = 0;
	freeList = id;
	count -= 1;
}

void HTree::refresh( int id, bool keepEnlarged )
{
	int a = child1[id], b = child2[id];
	box[id] = box_union( box[a], box[b] );
	cat[id] = cat[a] | cat[b];
	height[id] = 1 + imax( height[a], height[b] );
	if ( keepEnlarged )
		flags[id] |= ( flags[a] | flags[b] ) & PT_ENLARGED;
	leaves[id] = leaves[a] + leaves[b];
}

// :187-328 b2FindBestSibling
int HTree::best_sibling( float4 d ) const
{
	float2 centerD = box_center( d );
	float areaD = perimeter( d );
	int index = root;
	float4 rootBox = box[index];
	float areaBase = perimeter( rootBox );
	float directCost = perimeter( box_union( rootBox, d ) );
	float inherited = 0.0f;
	int best = index;
	float bestCost = directCost;
	while ( height[index] > 0 )
	{
		int c1 = child1[index], c2 = child2[index];
		float cost = directCost + inherited;
		if ( cost < bestCost )
		{
			best = index;
			bestCost = cost;
		}
		inherited += directCost - areaBase;
		bool leaf1 = height[c1] == 0, leaf2 = height[c2] == 0;
		float lower1 = FLT_MAX, area1 = 0.0f;
		float4 box1 = box[c1];
		float direct1 = perimeter( box_union( box1, d ) );
		if ( leaf1 )
		{
			float cost1 = direct1 + inherited;
			if ( cost1 < bestCost )
			{
				best = c1;
				bestCost = cost1;
			}
		}
		else
		{
			area1 = perimeter( box1 );
			float t = areaD - area1;
			lower1 = inherited + direct1 + ( t < 0.0f ? t : 0.0f );
		}
		float lower2 = FLT_MAX, area2 = 0.0f;
		float4 box2 = box[c2];
		float direct2 = perimeter( box_union( box2, d ) );
		if ( leaf2 )
		{
			float cost2 = direct2 + inherited;
			if ( cost2 < bestCost )
			{
				best = c2;
				bestCost = cost2;
			}
		}
		else
		{
			area2 = perimeter( box2 );
			float t = areaD - area2;
			lower2 = inherited + direct2 + ( t < 0.0f ? t : 0.0f );
		}
		if ( leaf1 && leaf2 )
			break;
		if ( bestCost <= lower1 && bestCost <= lower2 )
			break;
		if ( lower1 == lower2 && !leaf1 )
		{
			float2 m1 = box_center( box1 ), m2 = box_center( box2 );
			float dx1 = m1.x - centerD.x, dy1 = m1.y - centerD.y;
			float dx2 = m2.x - centerD.x, dy2 = m2.y - centerD.y;
			lower1 = dx1 * dx1 + dy1 * dy1;
			lower2 = dx2 * dx2 + dy2 * dy2;
		}
		if ( lower1 < lower2 && !leaf1 )
		{
			index = c1;
			areaBase = area1;
			directCost = direct1;
		}
		else
		{
			index = c2;
			areaBase = area2;
			directCost = direct2;
		}
	}
	return best;
}

// One exchange of b2RotateNodes (:338-623): `top`, a child of `a`, trades
// places with `g`, a child of a's other child `low`; `low` keeps `keep`.
void HTree::swap_in( int a, int top, int low, int g, int keep, int topSlot, int lowSlot, float4 lowBox )
{
	( topSlot == 1 ? child1 : child2 )[a] = g;
	( lowSlot == 1 ? child1 : child2 )[low] = top;
	parent[top] = low;
	parent[g] = a;
	box[low] = lowBox;
	height[low] = 1 + imax( height[top], height[keep] );
	height[a] = 1 + imax( height[low], height[g] );
	cat[low] = cat[top] | cat[keep];
	cat[a] = cat[low] | cat[g];
	flags[low] |= ( flags[top] | flags[keep] ) & PT_ENLARGED;
	flags[a] |= ( flags[low] | flags[g] ) & PT_ENLARGED;
	leaves[low] = leaves[top] + leaves[keep];
}

// :338-623 b2RotateNodes
void HTree::rotate( int iA )
{
	if ( height[iA] < 2 )
		return;
	int iB = child1[iA], iC = child2[iA];
	if ( height[iB] == 0 )
	{
		int iF = child1[iC], iG = child2[iC];
		float base = perimeter( box[iC] );
		float4 bg = box_union( box[iB], box[iG] );
		float costBF = perimeter( bg );
		float4 bf = box_union( box[iB], box[iF] );
		float costBG = perimeter( bf );
		if ( base < costBF && base < costBG )
			return;
		if ( costBF < costBG )
			swap_in( iA, iB, iC, iF, iG, 1, 1, bg );
		else
			swap_in( iA, iB, iC, iG, iF, 1, 2, bf );
		return;
	}
	if ( height[iC] == 0 )
	{
		int iD = child1[iB], iE = child2[iB];
		float base = perimeter( box[iB] );
		float4 ce = box_union( box[iC], box[iE] );
		float costCD = perimeter( ce );
		float4 cd = box_union( box[iC], box[iD] );
		float costCE = perimeter( cd );
		if ( base < costCD && base < costCE )
			return;
		if ( costCD < costCE )
			swap_in( iA, iC, iB, iD, iE, 2, 1, ce );
		else
			swap_in( iA, iC, iB, iE, iD, 2, 2, cd );
		return;
	}
	int iD = child1[iB], iE = child2[iB], iF = child1[iC], iG = child2[iC];
	float areaB = perimeter( box[iB] ), areaC = perimeter( box[iC] );
	float best = areaB + areaC;
	int choice = 0;
	float4 bg = box_union( box[iB], box[iG] );
	float c = areaB + perimeter( bg );
	if ( c < best )
	{
		choice = 1;
		best = c;
	}
	float4 bf = box_union( box[iB], box[iF] );
	c = areaB + perimeter( bf );
	if ( c < best )
	{
		choice = 2;
		best = c;
	}
	float4 ce = box_union( box[iC], box[iE] );
	c = areaC + perimeter( ce );
	if ( c < best )
	{
		choice = 3;
		best = c;
	}
	float4 cd = box_union( box[iC], box[iD] );
	c = areaC + perimeter( cd );
	if ( c < best )
		choice = 4;
	if ( choice == 1 )
		swap_in( iA, iB, iC, iF, iG, 1, 1, bg );
	else if ( choice == 2 )
		swap_in( iA, iB, iC, iG, iF, 1, 2, bf );
	else if ( choice == 3 )
		swap_in( iA, iC, iB, iD, iE, 2, 1, ce );
	else if ( choice == 4 )
		swap_in( iA, iC, iB, iE, iD, 2, 2, cd );
}

// :625-699 b2InsertLeaf: new parent (sibling child1, leaf child2), then the
// ancestors refreshed bottom up, rotated when asked
void HTree::insert_leaf( int leaf, bool shouldRotate )
{
	if ( root == -1 )
	{
		root = leaf;
		parent[leaf] = -1;
		return;
	}
	float4 leafBox = box[leaf];
	int sibling = best_sibling( leafBox );
	int oldParent = parent[sibling];
	int np = alloc_node();
	parent[np] = oldParent;
	box[np] = box_union( leafBox, box[sibling] );
	cat[np] = cat[leaf] | cat[sibling];
	height[np] = height[sibling] + 1;
	child1[np] = sibling;
	child2[np] = leaf;
	leaves[np] = leaves[sibling] + leaves[leaf];
	if ( oldParent != -1 )
	{
		if ( child1[oldParent] == sibling )
			child1[oldParent] = np;
		else
			child2[oldParent] = np;
	}
	else
		root = np;
	parent[sibling] = np;
	parent[leaf] = np;
	for ( int i = parent[leaf]; i != -1; i = parent[i] )
	{
		refresh( i, true );
		if ( shouldRotate )
			rotate( i );
	}
}

// :701-768 b2RemoveLeaf
void HTree::remove_leaf( int leaf )
{
	if ( leaf == root )
	{
		root = -1;
		return;
	}
	int p = parent[leaf];
	int gp = parent[p];
	int sibling = child1[p] == leaf ? child2[p] : child1[p];
	if ( gp != -1 )
	{
		if ( child1[gp] == p )
			child1[gp] = sibling;
		else
			child2[gp] = sibling;
		parent[sibling] = gp;
		free_node( p );
		for ( int i = gp; i != -1; i = parent[i] )
			refresh( i, false );
	}
	else
	{
		root = sibling;
		parent[sibling] = -1;
		free_node( p );
	}
}

// :770-792
int HTree::create_proxy( float4 aabb, unsigned long long category, int shapeId )
{
	int id = alloc_node();
	box[id] = aabb;
	shape[id] = shapeId;
	cat[id] = category;
	height[id] = 0;
	flags[id] = PT_ALLOCATED | PT_LEAF;
	leaves[id] = 1;
	insert_leaf( id, true );
	proxyCount += 1;
	return id;
}

// :794-804
void HTree::destroy_proxy( int proxyId )
{
	remove_leaf( proxyId );
	free_node( proxyId );
	proxyCount -= 1;
}

// :811-825 (re-insert, no rotations)
void HTree::move_proxy( int proxyId, float4 aabb )
{
	remove_leaf( proxyId );
	box[proxyId] = aabb;
	insert_leaf( proxyId, false );
}

// :868-891
void HTree::set_category( int proxyId, unsigned long long category )
{
	cat[proxyId] = category;
	for ( int p = parent[proxyId]; p != -1; p = parent[p] )
		cat[p] = cat[child1[p]] | cat[child2[p]];
}

// :1114-1170: stack of child1 then child2, so child2's subtree comes first;
// a category of zero is never visited
void HTree::visit_order( std::vector<int>& out ) const
{
	out.clear();
	if ( root == -1 )
		return;
	std::vector<int> stack;
	stack.push_back( root );
	while ( !stack.empty() )
	{
		int id = stack.back();
		stack.pop_back();
		if ( cat[id] == 0ull )
			continue;
		if ( flags[id] & PT_LEAF )
		{
			out.push_back( shape[id] );
			continue;
		}
		stack.push_back( child1[id] );
		stack.push_back( child2[id] );
	}
}
