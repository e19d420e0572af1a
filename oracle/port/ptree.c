// The reference's broadphase tree, restated (see ptree.h). TEST
// INFRASTRUCTURE (oracle). Reference file: packages/forge2d/third_party/
// box2d/src/dynamic_tree.c (v3.1.1); each function cites the lines it
// follows. Every float operation keeps the reference's operand order, since
// the tree's shape decides orders that the results depend on.
#include "ptree.h"

#include <float.h>
#include <stdlib.h>
#include <string.h>

static float perimeter( box2 a )
{
	// aabb.h:11-16 b2Perimeter
	float wx = a.hi.x - a.lo.x;
	float wy = a.hi.y - a.lo.y;
	return 2.0f * ( wx + wy );
}

static v2 box_center( box2 a )
{
	return V( 0.5f * ( a.lo.x + a.hi.x ), 0.5f * ( a.lo.y + a.hi.y ) );
}

static int max_int( int a, int b )
{
	return a > b ? a : b;
}

// :80-108 b2DynamicTree_Create: 16 nodes, all on the free list in order
void rt_init( RTree* t )
{
	memset( t, 0, sizeof( *t ) );
	t->root = P_NULL;
	t->cap = 16;
	t->nodes = calloc( (size_t)t->cap, sizeof( RNode ) );
	for ( int i = 0; i < t->cap; ++i )
		t->nodes[i].parent = i + 1 < t->cap ? i + 1 : P_NULL;
	t->freeList = 0;
}

void rt_release_all( RTree* t )
{
	free( t->nodes );
	free( t->rbNode );
	free( t->rbCenter );
	memset( t, 0, sizeof( *t ) );
	t->root = P_NULL;
}

// :122-158 b2AllocateNode: pop the free list; an empty list grows the pool
// by half, the new nodes chained in ascending order
static int node_alloc( RTree* t )
{
	if ( t->freeList == P_NULL )
	{
		int old = t->cap;
		t->cap = old + ( old >> 1 );
		t->nodes = realloc( t->nodes, sizeof( RNode ) * (size_t)t->cap );
		memset( t->nodes + old, 0, sizeof( RNode ) * (size_t)( t->cap - old ) );
		for ( int i = t->count; i < t->cap; ++i )
			t->nodes[i].parent = i + 1 < t->cap ? i + 1 : P_NULL;
		t->freeList = t->count;
	}
	int id = t->freeList;
	RNode* n = t->nodes + id;
	t->freeList = n->parent;
	memset( n, 0, sizeof( *n ) );
	n->category = P_DEFAULT_CATEGORY;
	n->child1 = P_NULL;
	n->child2 = P_NULL;
	n->shape = P_NULL;
	n->parent = P_NULL;
	n->flags = RN_ALLOCATED;
	t->count += 1;
	return id;
}

// :160-167 b2FreeNode: push on the free list
static void node_free( RTree* t, int id )
{
	t->nodes[id].parent = t->freeList;
	t->nodes[id].flags = 0;
	t->freeList = id;
	t->count -= 1;
}

// refresh an internal node from its children: box, category, height and
// the enlarged bit
static void refresh( RTree* t, int id, int keepEnlarged )
{
	RNode* n = t->nodes + id;
	const RNode* c1 = t->nodes + n->child1;
	const RNode* c2 = t->nodes + n->child2;
	n->aabb = boxUnion( c1->aabb, c2->aabb );
	n->category = c1->category | c2->category;
	n->height = 1 + max_int( c1->height, c2->height );
	if ( keepEnlarged )
		n->flags |= ( c1->flags | c2->flags ) & RN_ENLARGED;
}

// :187-328 b2FindBestSibling: one greedy descent, choosing between making a
// new parent here and descending into the child whose lower-bound cost is
// smaller (centre distance breaks an exact tie)
static int best_sibling( const RTree* t, box2 boxD )
{
	v2 centerD = box_center( boxD );
	float areaD = perimeter( boxD );
	const RNode* nodes = t->nodes;
	int index = t->root;
	box2 rootBox = nodes[index].aabb;
	float areaBase = perimeter( rootBox );
	float directCost = perimeter( boxUnion( rootBox, boxD ) );
	float inheritedCost = 0.0f;
	int best = index;
	float bestCost = directCost;
	while ( nodes[index].height > 0 )
	{
		int c1 = nodes[index].child1, c2 = nodes[index].child2;
		float cost = directCost + inheritedCost;
		if ( cost < bestCost )
		{
			best = index;
			bestCost = cost;
		}
		inheritedCost += directCost - areaBase;
		int leaf1 = nodes[c1].height == 0, leaf2 = nodes[c2].height == 0;

		float lower1 = FLT_MAX;
		box2 box1 = nodes[c1].aabb;
		float direct1 = perimeter( boxUnion( box1, boxD ) );
		float area1 = 0.0f;
		if ( leaf1 )
		{
			float cost1 = direct1 + inheritedCost;
			if ( cost1 < bestCost )
			{
				best = c1;
				bestCost = cost1;
			}
		}
		else
		{
			area1 = perimeter( box1 );
			lower1 = inheritedCost + direct1 + fminp( areaD - area1, 0.0f );
		}

		float lower2 = FLT_MAX;
		box2 box2v = nodes[c2].aabb;
		float direct2 = perimeter( boxUnion( box2v, boxD ) );
		float area2 = 0.0f;
		if ( leaf2 )
		{
			float cost2 = direct2 + inheritedCost;
			if ( cost2 < bestCost )
			{
				best = c2;
				bestCost = cost2;
			}
		}
		else
		{
			area2 = perimeter( box2v );
			lower2 = inheritedCost + direct2 + fminp( areaD - area2, 0.0f );
		}

		if ( leaf1 && leaf2 )
			break;
		if ( bestCost <= lower1 && bestCost <= lower2 )
			break;
		if ( lower1 == lower2 && leaf1 == 0 )
		{
			v2 d1 = sub( box_center( box1 ), centerD );
			v2 d2 = sub( box_center( box2v ), centerD );
			lower1 = d1.x * d1.x + d1.y * d1.y;
			lower2 = d2.x * d2.x + d2.y * d2.y;
		}
		if ( lower1 < lower2 && leaf1 == 0 )
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

// swap grandchild g (under `low`, the child of a being rebuilt) with the
// other child `top` of a: `low` keeps its other child `keep`. `topSlot` and
// `lowSlot` say which child pointer (1 or 2) is rewritten. (:338-623, the
// four swaps of b2RotateNodes share this form.)
static void swap_nodes( RTree* t, int a, int top, int low, int g, int keep, int topSlot, int lowSlot, box2 lowBox )
{
	RNode* nodes = t->nodes;
	if ( topSlot == 1 )
		nodes[a].child1 = g;
	else
		nodes[a].child2 = g;
	if ( lowSlot == 1 )
		nodes[low].child1 = top;
	else
		nodes[low].child2 = top;
	nodes[top].parent = low;
	nodes[g].parent = a;
	nodes[low].aabb = lowBox;
	nodes[low].height = 1 + max_int( nodes[top].height, nodes[keep].height );
	nodes[a].height = 1 + max_int( nodes[low].height, nodes[g].height );
	nodes[low].category = nodes[top].category | nodes[keep].category;
	nodes[a].category = nodes[low].category | nodes[g].category;
	nodes[low].flags |= ( nodes[top].flags | nodes[keep].flags ) & RN_ENLARGED;
	nodes[a].flags |= ( nodes[low].flags | nodes[g].flags ) & RN_ENLARGED;
}

// :338-623 b2RotateNodes: with A = (B, C), try swapping B or C with a
// grandchild on the other side when that lowers the summed perimeters
static void rotate_nodes( RTree* t, int iA )
{
	RNode* nodes = t->nodes;
	if ( nodes[iA].height < 2 )
		return;
	int iB = nodes[iA].child1, iC = nodes[iA].child2;
	if ( nodes[iB].height == 0 )
	{
		int iF = nodes[iC].child1, iG = nodes[iC].child2;
		float costBase = perimeter( nodes[iC].aabb );
		box2 aabbBG = boxUnion( nodes[iB].aabb, nodes[iG].aabb );
		float costBF = perimeter( aabbBG );
		box2 aabbBF = boxUnion( nodes[iB].aabb, nodes[iF].aabb );
		float costBG = perimeter( aabbBF );
		if ( costBase < costBF && costBase < costBG )
			return;
		if ( costBF < costBG )
			swap_nodes( t, iA, iB, iC, iF, iG, 1, 1, aabbBG );
		else
			swap_nodes( t, iA, iB, iC, iG, iF, 1, 2, aabbBF );
	}
	else if ( nodes[iC].height == 0 )
	{
		int iD = nodes[iB].child1, iE = nodes[iB].child2;
		float costBase = perimeter( nodes[iB].aabb );
		box2 aabbCE = boxUnion( nodes[iC].aabb, nodes[iE].aabb );
		float costCD = perimeter( aabbCE );
		box2 aabbCD = boxUnion( nodes[iC].aabb, nodes[iD].aabb );
		float costCE = perimeter( aabbCD );
		if ( costBase < costCD && costBase < costCE )
			return;
		if ( costCD < costCE )
			swap_nodes( t, iA, iC, iB, iD, iE, 2, 1, aabbCE );
		else
			swap_nodes( t, iA, iC, iB, iE, iD, 2, 2, aabbCD );
	}
	else
	{
		int iD = nodes[iB].child1, iE = nodes[iB].child2;
		int iF = nodes[iC].child1, iG = nodes[iC].child2;
		float areaB = perimeter( nodes[iB].aabb );
		float areaC = perimeter( nodes[iC].aabb );
		float best = areaB + areaC;
		int choice = 0;
		box2 aabbBG = boxUnion( nodes[iB].aabb, nodes[iG].aabb );
		float costBF = areaB + perimeter( aabbBG );
		if ( costBF < best )
		{
			choice = 1;
			best = costBF;
		}
		box2 aabbBF = boxUnion( nodes[iB].aabb, nodes[iF].aabb );
		float costBG = areaB + perimeter( aabbBF );
		if ( costBG < best )
		{
			choice = 2;
			best = costBG;
		}
		box2 aabbCE = boxUnion( nodes[iC].aabb, nodes[iE].aabb );
		float costCD = areaC + perimeter( aabbCE );
		if ( costCD < best )
		{
			choice = 3;
			best = costCD;
		}
		box2 aabbCD = boxUnion( nodes[iC].aabb, nodes[iD].aabb );
		float costCE = areaC + perimeter( aabbCD );
		if ( costCE < best )
			choice = 4;
		switch ( choice )
		{
			case 1:
				swap_nodes( t, iA, iB, iC, iF, iG, 1, 1, aabbBG );
				break;
			case 2:
				swap_nodes( t, iA, iB, iC, iG, iF, 1, 2, aabbBF );
				break;
			case 3:
				swap_nodes( t, iA, iC, iB, iD, iE, 2, 1, aabbCE );
				break;
			case 4:
				swap_nodes( t, iA, iC, iB, iE, iD, 2, 2, aabbCD );
				break;
			default:
				break;
		}
	}
}

// :625-699 b2InsertLeaf: a new parent joins the leaf and its best sibling
// (sibling child1, leaf child2), then the ancestors are refreshed bottom up,
// each rotated when `shouldRotate`
static void insert_leaf( RTree* t, int leaf, int shouldRotate )
{
	if ( t->root == P_NULL )
	{
		t->root = leaf;
		t->nodes[leaf].parent = P_NULL;
		return;
	}
	box2 leafBox = t->nodes[leaf].aabb;
	int sibling = best_sibling( t, leafBox );
	int oldParent = t->nodes[sibling].parent;
	int np = node_alloc( t );
	RNode* nodes = t->nodes;
	nodes[np].parent = oldParent;
	nodes[np].aabb = boxUnion( leafBox, nodes[sibling].aabb );
	nodes[np].category = nodes[leaf].category | nodes[sibling].category;
	nodes[np].height = nodes[sibling].height + 1;
	nodes[np].child1 = sibling;
	nodes[np].child2 = leaf;
	if ( oldParent != P_NULL )
	{
		if ( nodes[oldParent].child1 == sibling )
			nodes[oldParent].child1 = np;
		else
			nodes[oldParent].child2 = np;
	}
	else
		t->root = np;
	nodes[sibling].parent = np;
	nodes[leaf].parent = np;
	for ( int index = nodes[leaf].parent; index != P_NULL; index = nodes[index].parent )
	{
		refresh( t, index, 1 );
		if ( shouldRotate )
			rotate_nodes( t, index );
	}
}

// :701-768 b2RemoveLeaf: the leaf's parent is freed, its sibling takes its
// place, and the ancestors are refreshed (enlarged bits left as they are)
static void remove_leaf( RTree* t, int leaf )
{
	if ( leaf == t->root )
	{
		t->root = P_NULL;
		return;
	}
	RNode* nodes = t->nodes;
	int parent = nodes[leaf].parent;
	int grand = nodes[parent].parent;
	int sibling = nodes[parent].child1 == leaf ? nodes[parent].child2 : nodes[parent].child1;
	if ( grand != P_NULL )
	{
		if ( nodes[grand].child1 == parent )
			nodes[grand].child1 = sibling;
		else
			nodes[grand].child2 = sibling;
		nodes[sibling].parent = grand;
		node_free( t, parent );
		for ( int index = grand; index != P_NULL; index = nodes[index].parent )
			refresh( t, index, 0 );
	}
	else
	{
		t->root = sibling;
		nodes[sibling].parent = P_NULL;
		node_free( t, parent );
	}
}

// :770-792 b2DynamicTree_CreateProxy (insert with rotations)
int rt_create_proxy( RTree* t, box2 aabb, uint64_t category, int shape )
{
	int id = node_alloc( t );
	RNode* n = t->nodes + id;
	n->aabb = aabb;
	n->shape = shape;
	n->category = category;
	n->height = 0;
	n->flags = RN_ALLOCATED | RN_LEAF;
	insert_leaf( t, id, 1 );
	t->proxyCount += 1;
	return id;
}

// :794-804
void rt_destroy_proxy( RTree* t, int proxyId )
{
	remove_leaf( t, proxyId );
	node_free( t, proxyId );
	t->proxyCount -= 1;
}

// :811-825 (re-insert without rotations)
void rt_move_proxy( RTree* t, int proxyId, box2 aabb )
{
	remove_leaf( t, proxyId );
	t->nodes[proxyId].aabb = aabb;
	insert_leaf( t, proxyId, 0 );
}

// :827-866 b2DynamicTree_EnlargeProxy: grow the ancestors' boxes until one
// already holds the new box, marking every ancestor enlarged
void rt_enlarge_proxy( RTree* t, int proxyId, box2 aabb )
{
	RNode* nodes = t->nodes;
	nodes[proxyId].aabb = aabb;
	int p = nodes[proxyId].parent;
	while ( p != P_NULL )
	{
		box2* b = &nodes[p].aabb;
		int changed = 0;
		if ( aabb.lo.x < b->lo.x )
		{
			b->lo.x = aabb.lo.x;
			changed = 1;
		}
		if ( aabb.lo.y < b->lo.y )
		{
			b->lo.y = aabb.lo.y;
			changed = 1;
		}
		if ( b->hi.x < aabb.hi.x )
		{
			b->hi.x = aabb.hi.x;
			changed = 1;
		}
		if ( b->hi.y < aabb.hi.y )
		{
			b->hi.y = aabb.hi.y;
			changed = 1;
		}
		nodes[p].flags |= RN_ENLARGED;
		p = nodes[p].parent;
		if ( !changed )
			break;
	}
	while ( p != P_NULL && ( nodes[p].flags & RN_ENLARGED ) == 0 )
	{
		nodes[p].flags |= RN_ENLARGED;
		p = nodes[p].parent;
	}
}

// :868-891 b2DynamicTree_SetCategoryBits: the leaf and every ancestor
void rt_set_category( RTree* t, int proxyId, uint64_t category )
{
	RNode* nodes = t->nodes;
	nodes[proxyId].category = category;
	for ( int p = nodes[proxyId].parent; p != P_NULL; p = nodes[p].parent )
		nodes[p].category = nodes[nodes[p].child1].category | nodes[nodes[p].child2].category;
}

// :1114-1170 b2DynamicTree_Query: explicit stack, child1 pushed before child2
// (so child2's subtree is visited first); the stack lives on the C stack
// and moves to the heap only for trees deeper than it holds
void rt_query( const RTree* t, box2 aabb, uint64_t maskBits, rt_visit_fn fn, void* context )
{
	if ( t->count == 0 || t->root == P_NULL )
		return;
	int local[256];
	int* stack = local;
	int stackCap = 256, sp = 0;
	stack[sp++] = t->root;
	while ( sp > 0 )
	{
		int id = stack[--sp];
		const RNode* n = t->nodes + id;
		if ( boxOverlaps( n->aabb, aabb ) && ( n->category & maskBits ) != 0 )
		{
			if ( n->flags & RN_LEAF )
			{
				if ( fn( id, n->shape, context ) == 0 )
					break;
			}
			else
			{
				if ( sp + 2 > stackCap )
				{
					int* bigger = malloc( sizeof( int ) * (size_t)stackCap * 2 );
					memcpy( bigger, stack, sizeof( int ) * (size_t)sp );
					if ( stack != local )
						free( stack );
					stack = bigger;
					stackCap *= 2;
				}
				stack[sp++] = n->child1;
				stack[sp++] = n->child2;
			}
		}
	}
	if ( stack != local )
		free( stack );
}

static int cas_lower( float* addr, float v )
{
	int* ia = (int*)addr;
	int old = __atomic_load_n( ia, __ATOMIC_RELAXED );
	for ( ;; )
	{
		float cur;
		memcpy( &cur, &old, sizeof( cur ) );
		if ( !( v < cur ) )
			return 0;
		int nv;
		memcpy( &nv, &v, sizeof( nv ) );
		if ( __atomic_compare_exchange_n( ia, &old, nv, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED ) )
			return 1;
	}
}

static int cas_upper( float* addr, float v )
{
	int* ia = (int*)addr;
	int old = __atomic_load_n( ia, __ATOMIC_RELAXED );
	for ( ;; )
	{
		float cur;
		memcpy( &cur, &old, sizeof( cur ) );
		if ( !( cur < v ) )
			return 0;
		int nv;
		memcpy( &nv, &v, sizeof( nv ) );
		if ( __atomic_compare_exchange_n( ia, &old, nv, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED ) )
			return 1;
	}
}

// Many b2DynamicTree_EnlargeProxy calls at once (proxy ids and boxes in
// `count` rows). The serial calls leave every ancestor of an enlarged leaf
// marked, with its old box joined with the new boxes of the leaves below it,
// whatever their order; here each leaf climbs with compare-and-swap unions
// and stops at an ancestor that already held its box and was already
// marked (the thread that marked it carries the climb on), which gives the
// same boxes and marks.
void rt_enlarge_many( RTree* t, const int* proxies, const box2* boxes, int count )
{
	RNode* nodes = t->nodes;
#pragma omp parallel for schedule( dynamic, 256 )
	for ( int k = 0; k < count; ++k )
	{
		int leaf = proxies[k];
		box2 b = boxes[k];
		nodes[leaf].aabb = b;
		int p = nodes[leaf].parent;
		while ( p != P_NULL )
		{
			box2* pb = &nodes[p].aabb;
			int changed = cas_lower( &pb->lo.x, b.lo.x );
			changed |= cas_lower( &pb->lo.y, b.lo.y );
			changed |= cas_upper( &pb->hi.x, b.hi.x );
			changed |= cas_upper( &pb->hi.y, b.hi.y );
			int old = __atomic_fetch_or( &nodes[p].flags, RN_ENLARGED, __ATOMIC_RELAXED );
			if ( !changed && ( old & RN_ENLARGED ) )
				break;
			p = nodes[p].parent;
		}
	}
}

// :1426-1552 b2PartitionMid: Hoare partition of the centres about the middle
// of their bounds along the longer axis; returns the left count (half the
// range when one side would be empty)
static int partition_mid( int* idx, v2* cen, int count )
{
	if ( count <= 2 )
		return count / 2;
	v2 lo = cen[0], hi = cen[0];
	for ( int i = 1; i < count; ++i )
	{
		lo = vmin( lo, cen[i] );
		hi = vmax( hi, cen[i] );
	}
	v2 d = sub( hi, lo );
	int axisY = !( d.x > d.y );
	float pivot = axisY ? 0.5f * ( lo.y + hi.y ) : 0.5f * ( lo.x + hi.x );
	int i1 = 0, i2 = count;
	while ( i1 < i2 )
	{
		while ( i1 < i2 && ( axisY ? cen[i1].y : cen[i1].x ) < pivot )
			i1 += 1;
		while ( i1 < i2 && ( axisY ? cen[i2 - 1].y : cen[i2 - 1].x ) >= pivot )
			i2 -= 1;
		if ( i1 < i2 )
		{
			int ti = idx[i1];
			idx[i1] = idx[i2 - 1];
			idx[i2 - 1] = ti;
			v2 tc = cen[i1];
			cen[i1] = cen[i2 - 1];
			cen[i2 - 1] = tc;
			i1 += 1;
			i2 -= 1;
		}
	}
	if ( i1 > 0 && i1 < count )
		return i1;
	return count / 2;
}

// :1716-1870 b2BuildTree: top down over the gathered nodes, internal nodes
// allocated in pre-order (child1 side first), boxes filled bottom up
typedef struct BuildItem
{
	int node, childCount, start, split, end;
} BuildItem;

static int build_tree( RTree* t, int count )
{
	int* idx = t->rbNode;
	v2* cen = t->rbCenter;
	if ( count == 1 )
	{
		t->nodes[idx[0]].parent = P_NULL;
		return idx[0];
	}
	int stackCap = 64, top = 0;
	BuildItem* stack = malloc( sizeof( BuildItem ) * (size_t)stackCap );
	stack[0].node = node_alloc( t );
	stack[0].childCount = -1;
	stack[0].start = 0;
	stack[0].end = count;
	stack[0].split = partition_mid( idx, cen, count );
	for ( ;; )
	{
		BuildItem* item = stack + top;
		item->childCount += 1;
		if ( item->childCount == 2 )
		{
			refresh( t, item->node, 0 );
			if ( top == 0 )
				break;
			BuildItem* up = stack + top - 1;
			if ( up->childCount == 0 )
				t->nodes[up->node].child1 = item->node;
			else
				t->nodes[up->node].child2 = item->node;
			t->nodes[item->node].parent = up->node;
			top -= 1;
			continue;
		}
		int s = item->childCount == 0 ? item->start : item->split;
		int e = item->childCount == 0 ? item->split : item->end;
		if ( e - s == 1 )
		{
			int child = idx[s];
			if ( item->childCount == 0 )
				t->nodes[item->node].child1 = child;
			else
				t->nodes[item->node].child2 = child;
			t->nodes[child].parent = item->node;
			continue;
		}
		if ( top + 1 >= stackCap )
		{
			stackCap *= 2;
			stack = realloc( stack, sizeof( BuildItem ) * (size_t)stackCap );
		}
		int node = node_alloc( t ); // before `item` may move with the stack
		top += 1;
		BuildItem* next = stack + top;
		next->node = node;
		next->childCount = -1;
		next->start = s;
		next->end = e;
		next->split = s + partition_mid( idx + s, cen + s, e - s );
	}
	int root = stack[0].node;
	free( stack );
	return root;
}

// :1872-1989 b2DynamicTree_Rebuild: every enlarged internal node (every
// internal node when fullBuild) is freed, in pre-order; the leaves and the
// intact subtrees below them are gathered left to right and rebuilt over.
// Returns the number of gathered nodes.
int rt_rebuild( RTree* t, int fullBuild )
{
	if ( t->proxyCount == 0 || t->root == P_NULL )
		return 0;
	if ( t->proxyCount > t->rbCap )
	{
		t->rbCap = t->proxyCount + t->proxyCount / 2;
		t->rbNode = realloc( t->rbNode, sizeof( int ) * (size_t)t->rbCap );
		t->rbCenter = realloc( t->rbCenter, sizeof( v2 ) * (size_t)t->rbCap );
	}
	int count = 0;
	int stackCap = 256, sp = 0;
	int* stack = malloc( sizeof( int ) * (size_t)stackCap );
	int id = t->root;
	for ( ;; )
	{
		RNode* n = t->nodes + id;
		if ( n->height == 0 || ( ( n->flags & RN_ENLARGED ) == 0 && fullBuild == 0 ) )
		{
			t->rbNode[count] = id;
			t->rbCenter[count] = box_center( n->aabb );
			count += 1;
			n->parent = P_NULL;
		}
		else
		{
			int doomed = id;
			if ( sp + 1 > stackCap )
			{
				stackCap *= 2;
				stack = realloc( stack, sizeof( int ) * (size_t)stackCap );
			}
			stack[sp++] = n->child2;
			id = n->child1;
			node_free( t, doomed );
			continue;
		}
		if ( sp == 0 )
			break;
		id = stack[--sp];
	}
	free( stack );
	t->root = build_tree( t, count );
	return count;
}

void rt_leaf_ranks( const RTree* t, int* rank )
{
	if ( t->root == P_NULL )
		return;
	int stackCap = 256, sp = 0, next = 0;
	int* stack = malloc( sizeof( int ) * (size_t)stackCap );
	stack[sp++] = t->root;
	while ( sp > 0 )
	{
		int id = stack[--sp];
		const RNode* n = t->nodes + id;
		if ( n->flags & RN_LEAF )
		{
			rank[id] = next++;
			continue;
		}
		if ( sp + 2 > stackCap )
		{
			stackCap *= 2;
			stack = realloc( stack, sizeof( int ) * (size_t)stackCap );
		}
		stack[sp++] = n->child2;
		stack[sp++] = n->child1;
	}
	free( stack );
}
