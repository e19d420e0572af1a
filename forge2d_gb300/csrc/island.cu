// Islands, sleeping solver sets and waking on the device (island.c,
// solver_set.c; body.c:84-96, 1483-1508; joint.c:196-306; world.c:586-686,
// 1710-1740; solver.c:543-726, 1194-1220, 1473-1487, 1995-2048).
//
// Only worlds with sleeping enabled use this file. The reference keeps its
// islands with linked lists, union-find roots and swap-remove arrays whose
// orders decide which contacts re-enter the constraint graph, and in what
// order, when a set wakes; every function here follows those orders exactly
// and runs on one device thread (launch <<<1, 1>>>): the bookkeeping is
// serial by nature and touches few rows per step. The parallel phases of the
// step read the outcome through two flags: BF_ASLEEP on sleeping bodies (not
// integrated, not finalized) and CF_INACTIVE on contacts outside the awake
// set (not collided).
#include "dsort.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#include <cstddef>

#define ISL_NULL ( -1 )
#define F2D_TIME_TO_SLEEP 0.5f // constants.h:47
#define ISL_ERR_CAPACITY 1

__device__ __forceinline__ bool isl_static( const DWorld& w, int b )
{
	return body_type( w.bflags[b] ) == 0;
}

// ---------------------------------------------------------------------------
// constraint graph (constraint_graph.c:68-318), serial form
// ---------------------------------------------------------------------------
__device__ int isl_graph_add_contact( const DWorld& w, int c )
{
	int2 bd = w.cbody[c];
	int a = isl_static( w, bd.x ) ? -1 : bd.x, b = isl_static( w, bd.y ) ? -1 : bd.y;
	int color = F2D_OVERFLOW;
	if ( a >= 0 && b >= 0 )
	{
		unsigned used = w.colorMask[a] | w.colorMask[b];
		for ( int i = 0; i < F2D_OVERFLOW; ++i )
			if ( ( used & ( 1u << i ) ) == 0 )
			{
				color = i;
				break;
			}
		if ( color != F2D_OVERFLOW )
		{
			w.colorMask[a] |= 1u << color;
			w.colorMask[b] |= 1u << color;
		}
	}
	else
	{
		// no static contacts in colour 0
		int d = a >= 0 ? a : b;
		for ( int i = 1; i < F2D_OVERFLOW; ++i )
			if ( ( w.colorMask[d] & ( 1u << i ) ) == 0 )
			{
				color = i;
				break;
			}
		if ( color != F2D_OVERFLOW )
			w.colorMask[d] |= 1u << color;
	}
	w.ccolor[c] = color;
	if ( color == F2D_OVERFLOW )
	{
		int idx = w.sc->overflowCount;
		w.overflowList[idx] = c;
		w.coverflowIndex[c] = idx;
		w.sc->overflowCount = idx + 1;
	}
	return color;
}

__device__ void isl_graph_remove_contact( const DWorld& w, int c )
{
	int color = w.ccolor[c];
	if ( color == F2D_NULL )
		return;
	int2 bd = w.cbody[c];
	if ( color != F2D_OVERFLOW )
	{
		unsigned bit = 1u << color;
		if ( !isl_static( w, bd.x ) )
			w.colorMask[bd.x] &= ~bit;
		if ( !isl_static( w, bd.y ) )
			w.colorMask[bd.y] &= ~bit;
	}
	else
	{
		int idx = w.coverflowIndex[c];
		int last = w.sc->overflowCount - 1;
		if ( idx >= 0 && idx <= last )
		{
			if ( idx != last )
			{
				int moved = w.overflowList[last];
				w.overflowList[idx] = moved;
				w.coverflowIndex[moved] = idx;
			}
			w.sc->overflowCount = last;
		}
		w.coverflowIndex[c] = F2D_NULL;
	}
	w.ccolor[c] = F2D_NULL;
}

// joints may take colour 0 even against a static body (constraint_graph.c:214-267)
__device__ void isl_graph_add_joint( const DWorld& w, DIslands& I, int j )
{
	int2 jb = w.jbody[j];
	int a = isl_static( w, jb.x ) ? -1 : jb.x, b = isl_static( w, jb.y ) ? -1 : jb.y;
	int color = F2D_OVERFLOW;
	if ( a >= 0 && b >= 0 )
	{
		unsigned used = w.colorMask[a] | w.colorMask[b];
		for ( int c = 0; c < F2D_OVERFLOW; ++c )
			if ( ( used & ( 1u << c ) ) == 0 )
			{
				color = c;
				break;
			}
		if ( color != F2D_OVERFLOW )
		{
			w.colorMask[a] |= 1u << color;
			w.colorMask[b] |= 1u << color;
		}
	}
	else if ( a >= 0 || b >= 0 )
	{
		int d = a >= 0 ? a : b;
		for ( int c = 0; c < F2D_OVERFLOW; ++c )
			if ( ( w.colorMask[d] & ( 1u << c ) ) == 0 )
			{
				color = c;
				break;
			}
		if ( color != F2D_OVERFLOW )
			w.colorMask[d] |= 1u << color;
	}
	w.jcolor[j] = color;
	w.jcolorSet[j] = color == F2D_OVERFLOW ? 0 : ( a >= 0 ? 1 : 0 ) | ( b >= 0 ? 2 : 0 );
	if ( color == F2D_OVERFLOW )
	{
		int idx = w.sc->overflowJointCount;
		w.overflowJoints[idx] = j;
		I.jOverflowIndex[j] = idx;
		w.sc->overflowJointCount = idx + 1;
	}
}

__device__ void isl_graph_remove_joint( const DWorld& w, DIslands& I, int j )
{
	int color = w.jcolor[j];
	if ( color == F2D_NULL )
		return;
	int2 jb = w.jbody[j];
	if ( color != F2D_OVERFLOW )
	{
		// the bits its colouring set (the reference clears both bodies'
		// bits, constraint_graph.c:303-308, which differs only for a body
		// that was static when the joint was coloured and is not any more)
		unsigned bit = 1u << color;
		int set = w.jcolorSet[j];
		if ( set & 1 )
			w.colorMask[jb.x] &= ~bit;
		if ( set & 2 )
			w.colorMask[jb.y] &= ~bit;
	}
	else
	{
		int idx = I.jOverflowIndex[j];
		int last = w.sc->overflowJointCount - 1;
		if ( idx >= 0 && idx <= last )
		{
			if ( idx != last )
			{
				int moved = w.overflowJoints[last];
				w.overflowJoints[idx] = moved;
				I.jOverflowIndex[moved] = idx;
			}
			w.sc->overflowJointCount = last;
		}
		I.jOverflowIndex[j] = F2D_NULL;
	}
	w.jcolor[j] = F2D_NULL;
}

// ---------------------------------------------------------------------------
// id pools (id_pool.c:19-38) and sets
// ---------------------------------------------------------------------------
__device__ int isl_set_create( DIslands& I )
{
	int id = I.setFreeCount > 0 ? I.setFree[--I.setFreeCount] : I.setNext++;
	if ( id >= I.setCap )
	{
		I.error |= ISL_ERR_CAPACITY;
		id = I.setCap - 1;
	}
	DSet& s = I.sets[id];
	s.used = 1;
	s.headBody = s.tailBody = ISL_NULL;
	s.headContact = s.tailContact = ISL_NULL;
	s.headJoint = s.tailJoint = ISL_NULL;
	s.headIsland = s.tailIsland = ISL_NULL;
	s.bodyCount = s.contactCount = s.jointCount = s.islandCount = 0;
	return id;
}

__device__ void isl_set_destroy( DIslands& I, int id )
{
	I.sets[id].used = 0;
	I.setFree[I.setFreeCount++] = id;
}

// append to a sleeping set's list (its array order)
__device__ void isl_set_push_body( DIslands& I, int setId, int b )
{
	DSet& s = I.sets[setId];
	I.bSetNext[b] = ISL_NULL;
	if ( s.tailBody != ISL_NULL )
		I.bSetNext[s.tailBody] = b;
	else
		s.headBody = b;
	s.tailBody = b;
	s.bodyCount += 1;
	I.bSet[b] = setId;
}

__device__ void isl_set_push_contact( DIslands& I, int setId, int c )
{
	DSet& s = I.sets[setId];
	I.cSetNext[c] = ISL_NULL;
	if ( s.tailContact != ISL_NULL )
		I.cSetNext[s.tailContact] = c;
	else
		s.headContact = c;
	s.tailContact = c;
	s.contactCount += 1;
	I.cSet[c] = setId;
}

__device__ void isl_set_push_joint( DIslands& I, int setId, int j )
{
	DSet& s = I.sets[setId];
	I.jSetNext[j] = ISL_NULL;
	if ( s.tailJoint != ISL_NULL )
		I.jSetNext[s.tailJoint] = j;
	else
		s.headJoint = j;
	s.tailJoint = j;
	s.jointCount += 1;
	I.jSet[j] = setId;
}

__device__ void isl_set_push_island( DIslands& I, int setId, int id )
{
	DSet& s = I.sets[setId];
	I.islands[id].setNext = ISL_NULL;
	if ( s.tailIsland != ISL_NULL )
		I.islands[s.tailIsland].setNext = id;
	else
		s.headIsland = id;
	s.tailIsland = id;
	s.islandCount += 1;
	I.islands[id].setIndex = setId;
	I.islands[id].localIndex = s.islandCount - 1;
}

// the awake set's body array (swap-remove)
__device__ void isl_awake_add_body( const DWorld& w, DIslands& I, int b )
{
	int idx = I.awakeBodyCount++;
	I.awakeBodies[idx] = b;
	I.bLocal[b] = idx;
	I.bSet[b] = SET_AWAKE;
	w.bflags[b] &= ~BF_ASLEEP;
}

__device__ void isl_awake_remove_body( DIslands& I, int b )
{
	int idx = I.bLocal[b];
	int last = I.awakeBodyCount - 1;
	if ( idx != last )
	{
		int moved = I.awakeBodies[last];
		I.awakeBodies[idx] = moved;
		I.bLocal[moved] = idx;
	}
	I.awakeBodyCount = last;
	I.bLocal[b] = ISL_NULL;
}

// ---------------------------------------------------------------------------
// islands (island.c)
// ---------------------------------------------------------------------------
__device__ int isl_island_create( DIslands& I, int setId )
{
	int id = I.islandFreeCount > 0 ? I.islandFree[--I.islandFreeCount] : I.islandNext++;
	if ( id >= I.islandCap )
	{
		I.error |= ISL_ERR_CAPACITY;
		id = I.islandCap - 1;
	}
	DIsland& isl = I.islands[id];
	isl.headBody = isl.tailBody = ISL_NULL;
	isl.headContact = isl.tailContact = ISL_NULL;
	isl.headJoint = isl.tailJoint = ISL_NULL;
	isl.bodyCount = isl.contactCount = isl.jointCount = 0;
	isl.parent = ISL_NULL;
	isl.removeCount = 0;
	isl.setNext = ISL_NULL;
	if ( setId == SET_AWAKE )
	{
		isl.setIndex = SET_AWAKE;
		isl.localIndex = I.awakeIslandCount;
		I.awakeIslands[I.awakeIslandCount++] = id;
	}
	else
		isl_set_push_island( I, setId, id );
	return id;
}

// island.c:58-84 (awake islands only are destroyed)
__device__ void isl_island_destroy( DIslands& I, int id )
{
	if ( I.splitIslandId == id )
		I.splitIslandId = ISL_NULL;
	DIsland& isl = I.islands[id];
	int idx = isl.localIndex;
	int last = I.awakeIslandCount - 1;
	if ( idx != last )
	{
		int moved = I.awakeIslands[last];
		I.awakeIslands[idx] = moved;
		I.islands[moved].localIndex = idx;
	}
	I.awakeIslandCount = last;
	isl.setIndex = ISL_NULL;
	isl.localIndex = ISL_NULL;
	I.islandFree[I.islandFreeCount++] = id;
}

__device__ int isl_root( DIslands& I, int id )
{
	for ( int guard = 0; I.islands[id].parent != ISL_NULL && guard < I.islandCap; ++guard )
	{
		int parentId = I.islands[id].parent;
		int grand = I.islands[parentId].parent;
		if ( grand != ISL_NULL )
			I.islands[id].parent = grand;
		id = parentId;
	}
	return id;
}

__device__ void isl_add_contact( DIslands& I, int islandId, int c )
{
	DIsland& isl = I.islands[islandId];
	I.cIslandPrev[c] = ISL_NULL;
	I.cIslandNext[c] = ISL_NULL;
	if ( isl.headContact != ISL_NULL )
	{
		I.cIslandNext[c] = isl.headContact;
		I.cIslandPrev[isl.headContact] = c;
	}
	isl.headContact = c;
	if ( isl.tailContact == ISL_NULL )
		isl.tailContact = c;
	isl.contactCount += 1;
	I.cIsland[c] = islandId;
}

__device__ void isl_add_joint( DIslands& I, int islandId, int j )
{
	DIsland& isl = I.islands[islandId];
	I.jIslandPrev[j] = ISL_NULL;
	I.jIslandNext[j] = ISL_NULL;
	if ( isl.headJoint != ISL_NULL )
	{
		I.jIslandNext[j] = isl.headJoint;
		I.jIslandPrev[isl.headJoint] = j;
	}
	isl.headJoint = j;
	if ( isl.tailJoint == ISL_NULL )
		isl.tailJoint = j;
	isl.jointCount += 1;
	I.jIsland[j] = islandId;
}

__device__ void isl_wake_set( const DWorld& w, DIslands& I, int setId );

// island.c:116-218
__device__ void isl_link_contact( const DWorld& w, DIslands& I, int c )
{
	int2 bd = w.cbody[c];
	if ( I.bSet[bd.x] == SET_AWAKE && I.bSet[bd.y] >= SET_FIRST_SLEEPING )
		isl_wake_set( w, I, I.bSet[bd.y] );
	if ( I.bSet[bd.y] == SET_AWAKE && I.bSet[bd.x] >= SET_FIRST_SLEEPING )
		isl_wake_set( w, I, I.bSet[bd.x] );
	int idA = I.bIsland[bd.x], idB = I.bIsland[bd.y];
	if ( idA == idB )
	{
		isl_add_contact( I, idA, c );
		return;
	}
	int rootA = idA != ISL_NULL ? isl_root( I, idA ) : ISL_NULL;
	int rootB = idB != ISL_NULL ? isl_root( I, idB ) : ISL_NULL;
	if ( rootA != rootB && rootA != ISL_NULL && rootB != ISL_NULL )
		I.islands[rootB].parent = rootA;
	isl_add_contact( I, rootA != ISL_NULL ? rootA : rootB, c );
}

// island.c:221-261
__device__ void isl_unlink_contact( DIslands& I, int c )
{
	int id = I.cIsland[c];
	if ( id == ISL_NULL )
		return;
	DIsland& isl = I.islands[id];
	int prev = I.cIslandPrev[c], next = I.cIslandNext[c];
	if ( prev != ISL_NULL )
		I.cIslandNext[prev] = next;
	if ( next != ISL_NULL )
		I.cIslandPrev[next] = prev;
	if ( isl.headContact == c )
		isl.headContact = next;
	if ( isl.tailContact == c )
		isl.tailContact = prev;
	isl.contactCount -= 1;
	isl.removeCount += 1;
	I.cIsland[c] = I.cIslandPrev[c] = I.cIslandNext[c] = ISL_NULL;
}

__device__ void isl_merge_awake( DIslands& I );

// island.c:291-382
__device__ void isl_link_joint( const DWorld& w, DIslands& I, int j, bool merge )
{
	int2 jb = w.jbody[j];
	if ( I.bSet[jb.x] == SET_AWAKE && I.bSet[jb.y] >= SET_FIRST_SLEEPING )
		isl_wake_set( w, I, I.bSet[jb.y] );
	else if ( I.bSet[jb.y] == SET_AWAKE && I.bSet[jb.x] >= SET_FIRST_SLEEPING )
		isl_wake_set( w, I, I.bSet[jb.x] );
	int idA = I.bIsland[jb.x], idB = I.bIsland[jb.y];
	if ( idA == idB )
	{
		isl_add_joint( I, idA, j );
		return;
	}
	int rootA = idA != ISL_NULL ? isl_root( I, idA ) : ISL_NULL;
	int rootB = idB != ISL_NULL ? isl_root( I, idB ) : ISL_NULL;
	if ( rootA != rootB && rootA != ISL_NULL && rootB != ISL_NULL )
		I.islands[rootB].parent = rootA;
	isl_add_joint( I, rootA != ISL_NULL ? rootA : rootB, j );
	if ( merge )
		isl_merge_awake( I );
}

// island.c:429-528
// remap: move the members' island ids too (the step's merge has done that
// for all islands at once, k_isl_merge_remap)
__device__ void isl_merge_one( DIslands& I, int id, bool remap = true )
{
	DIsland& isl = I.islands[id];
	int rootId = isl.parent;
	DIsland& root = I.islands[rootId];
	if ( remap )
	{
		for ( int b = isl.headBody, g = 0; b != ISL_NULL && g < I.bodyCap; b = I.bIslandNext[b], ++g )
			I.bIsland[b] = rootId;
		for ( int c = isl.headContact, g = 0; c != ISL_NULL && g < I.contactCap; c = I.cIslandNext[c], ++g )
			I.cIsland[c] = rootId;
		for ( int j = isl.headJoint, g = 0; j != ISL_NULL && g < I.jointCap; j = I.jIslandNext[j], ++g )
			I.jIsland[j] = rootId;
	}
	I.bIslandNext[root.tailBody] = isl.headBody;
	I.bIslandPrev[isl.headBody] = root.tailBody;
	root.tailBody = isl.tailBody;
	root.bodyCount += isl.bodyCount;
	if ( root.headContact == ISL_NULL )
	{
		root.headContact = isl.headContact;
		root.tailContact = isl.tailContact;
		root.contactCount = isl.contactCount;
	}
	else if ( isl.headContact != ISL_NULL )
	{
		I.cIslandNext[root.tailContact] = isl.headContact;
		I.cIslandPrev[isl.headContact] = root.tailContact;
		root.tailContact = isl.tailContact;
		root.contactCount += isl.contactCount;
	}
	if ( root.headJoint == ISL_NULL )
	{
		root.headJoint = isl.headJoint;
		root.tailJoint = isl.tailJoint;
		root.jointCount = isl.jointCount;
	}
	else if ( isl.headJoint != ISL_NULL )
	{
		I.jIslandNext[root.tailJoint] = isl.headJoint;
		I.jIslandPrev[isl.headJoint] = root.tailJoint;
		root.tailJoint = isl.tailJoint;
		root.jointCount += isl.jointCount;
	}
	root.removeCount += isl.removeCount;
}

// island.c:539-600
__device__ void isl_merge_awake( DIslands& I )
{
	int n = I.awakeIslandCount;
	for ( int i = 0; i < n; ++i )
	{
		int id = I.awakeIslands[i];
		int root = isl_root( I, id );
		if ( root != id )
			I.islands[id].parent = root;
	}
	for ( int i = n - 1; i >= 0; --i )
	{
		int id = I.awakeIslands[i];
		if ( I.islands[id].parent == ISL_NULL )
			continue;
		isl_merge_one( I, id );
		isl_island_destroy( I, id );
	}
}

// island.c:602-832
__device__ void isl_split( const DWorld& w, DIslands& I, int baseId )
{
	DIsland& base = I.islands[baseId];
	if ( base.setIndex != SET_AWAKE || base.removeCount == 0 )
		return;
	int bodyCount = base.bodyCount;
	int index = 0;
	for ( int b = base.headBody, g = 0; b != ISL_NULL && g < I.bodyCap; b = I.bIslandNext[b], ++g )
	{
		I.seeds[index++] = b;
		I.bMark[b] = 0;
	}
	for ( int c = base.headContact, g = 0; c != ISL_NULL && g < I.contactCap; c = I.cIslandNext[c], ++g )
		I.cMark[c] = 0;
	for ( int j = base.headJoint, g = 0; j != ISL_NULL && g < I.jointCap; j = I.jIslandNext[j], ++g )
		I.jMark[j] = 0;
	isl_island_destroy( I, baseId );

	for ( int i = 0; i < bodyCount; ++i )
	{
		int seed = I.seeds[i];
		if ( I.bMark[seed] )
			continue;
		int sp = 0;
		I.stack[sp++] = seed;
		I.bMark[seed] = 1;
		int id = isl_island_create( I, SET_AWAKE );
		while ( sp > 0 )
		{
			int b = I.stack[--sp];
			DIsland& isl = I.islands[id];
			I.bIsland[b] = id;
			if ( isl.tailBody != ISL_NULL )
				I.bIslandNext[isl.tailBody] = b;
			I.bIslandPrev[b] = isl.tailBody;
			I.bIslandNext[b] = ISL_NULL;
			isl.tailBody = b;
			if ( isl.headBody == ISL_NULL )
				isl.headBody = b;
			isl.bodyCount += 1;

			for ( int key = I.bHeadContact[b], g = 0; key != ISL_NULL && g < I.contactCap; ++g )
			{
				int c = key >> 1, edge = key & 1;
				int4 e = I.cEdge[c];
				key = edge == 0 ? e.y : e.w;
				if ( I.cMark[c] )
					continue;
				if ( ( w.cflags[c] & CF_TOUCHING ) == 0 )
					continue;
				I.cMark[c] = 1;
				int2 bd = w.cbody[c];
				int other = edge == 0 ? bd.y : bd.x;
				if ( I.bMark[other] == 0 && I.bSet[other] != SET_STATIC )
				{
					if ( sp < I.bodyCap )
						I.stack[sp++] = other;
					I.bMark[other] = 1;
				}
				I.cIsland[c] = id;
				if ( isl.tailContact != ISL_NULL )
					I.cIslandNext[isl.tailContact] = c;
				I.cIslandPrev[c] = isl.tailContact;
				I.cIslandNext[c] = ISL_NULL;
				isl.tailContact = c;
				if ( isl.headContact == ISL_NULL )
					isl.headContact = c;
				isl.contactCount += 1;
			}

			for ( int key = w.headJoint[b], g = 0; key != F2D_NULL && g < I.jointCap; ++g )
			{
				int j = key >> 1, edge = key & 1;
				key = w.jnext[2 * j + edge];
				if ( I.jMark[j] )
					continue;
				I.jMark[j] = 1;
				int2 jb = w.jbody[j];
				int other = edge == 0 ? jb.y : jb.x;
				if ( I.bSet[other] == SET_DISABLED )
					continue;
				if ( I.bMark[other] == 0 && I.bSet[other] == SET_AWAKE )
				{
					if ( sp < I.bodyCap )
						I.stack[sp++] = other;
					I.bMark[other] = 1;
				}
				I.jIsland[j] = id;
				if ( isl.tailJoint != ISL_NULL )
					I.jIslandNext[isl.tailJoint] = j;
				I.jIslandPrev[j] = isl.tailJoint;
				I.jIslandNext[j] = ISL_NULL;
				isl.tailJoint = j;
				if ( isl.headJoint == ISL_NULL )
					isl.headJoint = j;
				isl.jointCount += 1;
			}
		}
	}
}

// ---------------------------------------------------------------------------
// body contact edge lists (contact.c:240-283, 355-410)
// ---------------------------------------------------------------------------
__device__ void isl_edges_link( const DWorld& w, DIslands& I, int c )
{
	int2 bd = w.cbody[c];
	int4 e = make_int4( ISL_NULL, ISL_NULL, ISL_NULL, ISL_NULL );
	for ( int edge = 0; edge < 2; ++edge )
	{
		int b = edge == 0 ? bd.x : bd.y;
		int key = ( c << 1 ) | edge;
		int head = I.bHeadContact[b];
		if ( edge == 0 )
			e.y = head;
		else
			e.w = head;
		if ( head != ISL_NULL )
		{
			// the head is another contact's edge (bodies A and B differ)
			int4 he = I.cEdge[head >> 1];
			if ( head & 1 )
				he.z = key;
			else
				he.x = key;
			I.cEdge[head >> 1] = he;
		}
		I.bHeadContact[b] = key;
	}
	I.cEdge[c] = e;
}

__device__ void isl_edges_unlink( const DWorld& w, DIslands& I, int c )
{
	int2 bd = w.cbody[c];
	for ( int edge = 0; edge < 2; ++edge )
	{
		int4 e = I.cEdge[c];
		int prev = edge == 0 ? e.x : e.z;
		int next = edge == 0 ? e.y : e.w;
		if ( prev != ISL_NULL )
		{
			int4 pe = I.cEdge[prev >> 1];
			if ( prev & 1 )
				pe.w = next;
			else
				pe.y = next;
			I.cEdge[prev >> 1] = pe;
		}
		if ( next != ISL_NULL )
		{
			int4 ne = I.cEdge[next >> 1];
			if ( next & 1 )
				ne.z = prev;
			else
				ne.x = prev;
			I.cEdge[next >> 1] = ne;
		}
		int b = edge == 0 ? bd.x : bd.y;
		if ( I.bHeadContact[b] == ( ( c << 1 ) | edge ) )
			I.bHeadContact[b] = next;
	}
	I.cEdge[c] = make_int4( ISL_NULL, ISL_NULL, ISL_NULL, ISL_NULL );
}

// ---------------------------------------------------------------------------
// sleeping and waking (solver_set.c)
// ---------------------------------------------------------------------------
// solver_set.c:36-147
__device__ void isl_wake_set( const DWorld& w, DIslands& I, int setId )
{
	DSet s = I.sets[setId];
	for ( int b = s.headBody, g = 0; b != ISL_NULL && g < I.bodyCap; ++g )
	{
		int next = I.bSetNext[b];
		isl_awake_add_body( w, I, b );
		float4 fo = w.force[b];
		w.force[b] = make_float4( fo.x, fo.y, fo.z, 0.0f ); // sleep time reset
		w.vel[b] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );	  // b2_identityBodyState
		w.delta[b] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
		for ( int key = I.bHeadContact[b], k = 0; key != ISL_NULL && k < I.contactCap; ++k )
		{
			int c = key >> 1;
			int4 e = I.cEdge[c];
			key = ( key & 1 ) ? e.w : e.y;
			if ( I.cSet[c] != SET_DISABLED )
				continue;
			I.cSet[c] = SET_AWAKE;
			w.cflags[c] &= ~CF_INACTIVE;
		}
		b = next;
	}
	for ( int c = s.headContact, g = 0; c != ISL_NULL && g < I.contactCap; ++g )
	{
		int next = I.cSetNext[c];
		isl_graph_add_contact( w, c );
		I.cSet[c] = SET_AWAKE;
		w.cflags[c] &= ~CF_INACTIVE;
		c = next;
	}
	for ( int j = s.headJoint, g = 0; j != ISL_NULL && g < I.jointCap; ++g )
	{
		int next = I.jSetNext[j];
		isl_graph_add_joint( w, I, j );
		I.jSet[j] = SET_AWAKE;
		j = next;
	}
	for ( int id = s.headIsland, g = 0; id != ISL_NULL && g < I.islandCap; ++g )
	{
		int next = I.islands[id].setNext;
		DIsland& isl = I.islands[id];
		isl.setIndex = SET_AWAKE;
		isl.localIndex = I.awakeIslandCount;
		isl.setNext = ISL_NULL;
		I.awakeIslands[I.awakeIslandCount++] = id;
		id = next;
	}
	isl_set_destroy( I, setId );
}

// solver_set.c:156-414
__device__ void isl_try_sleep( const DWorld& w, DIslands& I, int islandId )
{
	if ( I.islands[islandId].removeCount > 0 )
		return;
	int sleepId = isl_set_create( I );
	DIsland& isl = I.islands[islandId];
	for ( int b = isl.headBody, g = 0; b != ISL_NULL && g < I.bodyCap; ++g )
	{
		if ( I.bMoveIndex[b] != ISL_NULL )
		{
			I.moveAsleep[I.bMoveIndex[b]] = 1;
			I.bMoveIndex[b] = ISL_NULL;
		}
		isl_awake_remove_body( I, b );
		isl_set_push_body( I, sleepId, b );
		w.bflags[b] |= BF_ASLEEP;
		w.vel[b] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		w.delta[b] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
		for ( int key = I.bHeadContact[b], k = 0; key != ISL_NULL && k < I.contactCap; ++k )
		{
			int c = key >> 1, edge = key & 1;
			int4 e = I.cEdge[c];
			key = edge == 0 ? e.y : e.w;
			if ( I.cSet[c] == SET_DISABLED )
				continue;
			if ( w.ccolor[c] != F2D_NULL )
				continue;
			int2 bd = w.cbody[c];
			int other = edge == 0 ? bd.y : bd.x;
			if ( I.bSet[other] == SET_AWAKE )
				continue;
			I.cSet[c] = SET_DISABLED;
			w.cflags[c] |= CF_INACTIVE;
		}
		b = I.bIslandNext[b];
	}
	for ( int c = isl.headContact, g = 0; c != ISL_NULL && g < I.contactCap; ++g )
	{
		isl_graph_remove_contact( w, c );
		isl_set_push_contact( I, sleepId, c );
		w.cflags[c] |= CF_INACTIVE;
		c = I.cIslandNext[c];
	}
	for ( int j = isl.headJoint, g = 0; j != ISL_NULL && g < I.jointCap; ++g )
	{
		isl_graph_remove_joint( w, I, j );
		isl_set_push_joint( I, sleepId, j );
		j = I.jIslandNext[j];
	}
	int idx = isl.localIndex;
	int last = I.awakeIslandCount - 1;
	if ( idx != last )
	{
		int moved = I.awakeIslands[last];
		I.awakeIslands[idx] = moved;
		I.islands[moved].localIndex = idx;
	}
	I.awakeIslandCount = last;
	isl_set_push_island( I, sleepId, islandId );
	I.islands[islandId].localIndex = 0;
}

// solver_set.c:419-517
__device__ void isl_merge_sets( DIslands& I, int s1, int s2 )
{
	if ( I.sets[s1].bodyCount < I.sets[s2].bodyCount )
	{
		int t = s1;
		s1 = s2;
		s2 = t;
	}
	DSet src = I.sets[s2];
	for ( int b = src.headBody, g = 0; b != ISL_NULL && g < I.bodyCap; ++g )
	{
		int next = I.bSetNext[b];
		isl_set_push_body( I, s1, b );
		b = next;
	}
	for ( int c = src.headContact, g = 0; c != ISL_NULL && g < I.contactCap; ++g )
	{
		int next = I.cSetNext[c];
		isl_set_push_contact( I, s1, c );
		c = next;
	}
	for ( int j = src.headJoint, g = 0; j != ISL_NULL && g < I.jointCap; ++g )
	{
		int next = I.jSetNext[j];
		isl_set_push_joint( I, s1, j );
		j = next;
	}
	for ( int id = src.headIsland, g = 0; id != ISL_NULL && g < I.islandCap; ++g )
	{
		int next = I.islands[id].setNext;
		isl_set_push_island( I, s1, id );
		id = next;
	}
	isl_set_destroy( I, s2 );
}

// ---------------------------------------------------------------------------
// kernels (all <<<1, 1>>>)
// ---------------------------------------------------------------------------
// Bodies and joints created since the last step, in creation order
// (body.c:225-330 set and island; joint.c:196-306 set, graph and island).
__global__ void k_isl_create( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	for ( int i = 0; i < I.logCount; ++i )
	{
		int kind = (unsigned)I.log[i] >> 30;
		int id = I.log[i] & 0x3fffffff;
		if ( kind == 0 )
		{
			if ( id + 1 > I.bodyKnown )
				I.bodyKnown = id + 1;
			int f = w.bflags[id];
			I.bIsland[id] = I.bIslandPrev[id] = I.bIslandNext[id] = ISL_NULL;
			I.bHeadContact[id] = ISL_NULL;
			I.bMoveIndex[id] = ISL_NULL;
			I.bLocal[id] = ISL_NULL;
			int setId;
			if ( ( f & BF_ENABLED ) == 0 )
				setId = SET_DISABLED;
			else if ( body_type( f ) == 0 )
				setId = SET_STATIC;
			else if ( ( f & BF_ASLEEP ) == 0 )
				setId = SET_AWAKE;
			else
				setId = isl_set_create( I );
			if ( setId == SET_AWAKE )
				isl_awake_add_body( w, I, id );
			else if ( setId >= SET_FIRST_SLEEPING )
				isl_set_push_body( I, setId, id );
			else
				I.bSet[id] = setId;
			if ( setId >= SET_AWAKE )
			{
				int isl = isl_island_create( I, setId );
				I.bIsland[id] = isl;
				I.islands[isl].headBody = I.islands[isl].tailBody = id;
				I.islands[isl].bodyCount = 1;
			}
		}
		else
		{
			int2 jb = w.jbody[id];
			I.jIsland[id] = I.jIslandPrev[id] = I.jIslandNext[id] = ISL_NULL;
			I.jOverflowIndex[id] = ISL_NULL;
			int sa = I.bSet[jb.x], sb = I.bSet[jb.y];
			int maxSet = sa > sb ? sa : sb;
			w.jcolor[id] = F2D_NULL;
			if ( sa == SET_DISABLED || sb == SET_DISABLED )
				I.jSet[id] = SET_DISABLED;
			else if ( sa == SET_STATIC && sb == SET_STATIC )
				I.jSet[id] = SET_STATIC;
			else if ( sa == SET_AWAKE || sb == SET_AWAKE )
			{
				if ( maxSet >= SET_FIRST_SLEEPING )
					isl_wake_set( w, I, maxSet );
				I.jSet[id] = SET_AWAKE;
				isl_graph_add_joint( w, I, id );
			}
			else
			{
				isl_set_push_joint( I, maxSet, id );
				if ( sa != sb && sa >= SET_FIRST_SLEEPING && sb >= SET_FIRST_SLEEPING )
					isl_merge_sets( I, sa, sb );
			}
			if ( I.jSet[id] > SET_DISABLED )
				isl_link_joint( w, I, id, true );
		}
	}
	I.logCount = 0;
}

// New contacts of the step in creation order: set and body edge lists
// (contact.c:206-283). Native order is the new-pair key order; in parity
// mode, the order the id pool handed the planned ids out.
__global__ void k_isl_new_contacts( DWorld w, DIslands* Ip, int planMode )
{
	DIslands& I = *Ip;
	int n = w.sc->newPairCount;
	int F = w.sc->contactFreeCount;
	int base = w.sc->contactIdCount;
	int m = 0;
	for ( int r = 0; r < n; ++r )
	{
		int id;
		if ( planMode )
			id = w.newPairId[r];
		else
			id = r < F ? w.contactFree[F - 1 - r] : base + ( r - F );
		if ( id < 0 || id >= w.contactCap || ( w.cflags[id] & CF_USED ) == 0 )
			continue;
		I.order[m++] = id;
	}
	if ( planMode )
	{
		// rank = position in the LIFO pop order, then fresh ids ascending
		for ( int i = 1; i < m; ++i )
		{
			int v = I.order[i];
			long long rv = v >= base ? (long long)F + ( v - base ) : 0;
			if ( v < base )
				for ( int k = F - 1; k >= 0; --k )
					if ( w.contactFree[k] == v )
					{
						rv = F - 1 - k;
						break;
					}
			int j = i - 1;
			while ( j >= 0 )
			{
				int u = I.order[j];
				long long ru = u >= base ? (long long)F + ( u - base ) : 0;
				if ( u < base )
					for ( int k = F - 1; k >= 0; --k )
						if ( w.contactFree[k] == u )
						{
							ru = F - 1 - k;
							break;
						}
				if ( ru <= rv )
					break;
				I.order[j + 1] = u;
				j -= 1;
			}
			I.order[j + 1] = v;
		}
	}
	for ( int i = 0; i < m; ++i )
	{
		int c = I.order[i];
		int2 bd = w.cbody[c];
		bool awake = I.bSet[bd.x] == SET_AWAKE || I.bSet[bd.y] == SET_AWAKE;
		I.cSet[c] = awake ? SET_AWAKE : SET_DISABLED;
		I.cIsland[c] = I.cIslandPrev[c] = I.cIslandNext[c] = ISL_NULL;
		I.cMark[c] = 0;
		if ( !awake )
			w.cflags[c] |= CF_INACTIVE;
		isl_edges_link( w, I, c );
	}
}

// The step's contact state changes in contact-id order (world.c:586-686)
// with island links, unlinks and the wakes they cause, then the island
// merge that opens b2Solve (solver.c:1194-1199).
// A contact that begins touching between an awake and a sleeping body wakes
// the sleeping set inside the serial loop (island.c:116-130), and the woken
// contacts enter the colour graph between the step's own changes: such a
// step keeps the whole serial form below. Any other step colours in
// parallel (graph.cu) and takes the island changes apart: unlinks as one
// set removal (their order does not change the lists: removing and
// prepending commute), links serially.
__global__ void k_isl_op_check( DWorld w, DIslands* Ip )
{
	const DIslands& I = *Ip;
	int nOps = min( w.sc->opCount, w.opCap );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		if ( w.opKind[k] != 1 )
			continue;
		int2 bd = w.cbody[w.opContact[k]];
		if ( I.bSet[bd.x] >= SET_FIRST_SLEEPING || I.bSet[bd.y] >= SET_FIRST_SLEEPING )
			atomicOr( &Ip->serialOps, 1 );
	}
}

__global__ void k_isl_ops( DWorld w, DIslands* Ip, const int* gkind )
{
	DIslands& I = *Ip;
	if ( I.serialOps == 0 )
		return;
	I.linkCount = 0; // nothing for the parallel link kernels to sort
	int nOps = w.sc->opCount;
	if ( nOps > w.opCap )
		nOps = w.opCap;
	for ( int k = 0; k < nOps; ++k )
	{
		w.opDone[k] = 1; // nothing left for the parallel colouring
		int c = w.opContact[k];
		int kind = w.opKind[k];
		if ( kind == 0 )
		{
			// b2DestroyContact: edges, island, graph
			isl_edges_unlink( w, I, c );
			isl_unlink_contact( I, c );
			w.opColor[k] = w.ccolor[c];
			isl_graph_remove_contact( w, c );
		}
		else if ( kind == 1 )
		{
			w.cflags[c] |= CF_TOUCHING;
			isl_link_contact( w, I, c );
			w.opColor[k] = isl_graph_add_contact( w, c );
		}
		else
		{
			isl_unlink_contact( I, c );
			w.opColor[k] = w.ccolor[c];
			isl_graph_remove_contact( w, c );
		}
	}
	(void)gkind;
	w.sc->overflowOps = 0;
	w.sc->colorRounds = 1;
}

// Island merge at the start of b2Solve (island.c:539-600) in three parts:
// every awake island points at its root (parallel; roots never change), the
// islands that have a parent are listed in array order (scan), and one
// thread merges them into their roots from the last to the first, as the
// reference's reverse loop does.
__global__ void k_isl_merge_roots( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	int n = I.awakeIslandCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		int id = I.awakeIslands[i];
		int root = id;
		for ( int g = 0; I.islands[root].parent != ISL_NULL && g < I.islandCap; ++g )
			root = I.islands[root].parent;
		I.flag[i] = root != id ? 1 : 0;
		if ( root != id )
			I.islands[id].parent = root;
	}
}

__global__ void k_isl_list( DIslands* Ip, const int* count )
{
	DIslands& I = *Ip;
	int n = *count;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
		if ( I.flag[i] )
			I.list[I.pos[i]] = I.awakeIslands[i];
}

// island.c:539-600 members of merged islands: every body, contact and joint
// of an island that has a parent (a root, after k_isl_merge_roots) takes the
// root's id, all at once
__global__ void k_isl_merge_remap( DWorld w, DIslands* Ip )
{
	const DIslands& I = *Ip;
	if ( I.listCount == 0 )
		return;
	int nb = min( I.bodyKnown, I.bodyCap ), nc = w.sc->contactIdCount, nj = w.jointCount;
	int total = nb + nc + nj;
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x )
	{
		int* slot = k < nb ? I.bIsland + k : k < nb + nc ? I.cIsland + ( k - nb ) : I.jIsland + ( k - nb - nc );
		int id = *slot;
		if ( id == ISL_NULL )
			continue;
		int p = I.islands[id].parent;
		if ( p != ISL_NULL )
			*slot = p;
	}
}

__global__ void k_isl_merge_apply( DIslands* Ip )
{
	DIslands& I = *Ip;
	for ( int k = I.listCount - 1; k >= 0; --k )
	{
		int id = I.list[k];
		isl_merge_one( I, id, false );
		isl_island_destroy( I, id );
	}
}

// Split of the previous step's candidate, before the bodies are finalized
// (solver.c:1473-1487, 1700-1706); move-event slots in awake order.
__global__ void k_isl_split( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	if ( I.awakeBodyCount == 0 )
		return;
	if ( I.splitIslandId != ISL_NULL )
		isl_split( w, I, I.splitIslandId );
	I.splitIslandId = ISL_NULL;
}

// Move-event slots in awake order, cleared keep-awake bits and candidate.
__global__ void k_isl_move_slots( DIslands* Ip )
{
	DIslands& I = *Ip;
	int n = I.awakeBodyCount;
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
	{
		I.moveCount = n;
		I.candKey = 0ull;
	}
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		int b = I.awakeBodies[i];
		I.bMoveIndex[b] = i;
		I.moveBody[i] = b;
		I.moveAsleep[i] = 0;
	}
	int ni = I.awakeIslandCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x )
		I.islandBits[i] = 0;
}

// Keep-awake bits and the split candidate (solver.c:658-675): the first body
// in awake order with the largest sleep time wins, as one task context scans.
__global__ void k_isl_bits( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	int n = I.moveCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
	{
		int b = I.awakeBodies[i];
		float sleepTime = w.force[b].w;
		const DIsland& isl = I.islands[I.bIsland[b]];
		if ( sleepTime < F2D_TIME_TO_SLEEP )
			I.islandBits[isl.localIndex] = 1;
		else if ( isl.removeCount > 0 && sleepTime > 0.0f )
		{
			unsigned long long key =
				( (unsigned long long)__float_as_uint( sleepTime ) << 32 ) | (unsigned)( 0xffffffffu - (unsigned)i );
			atomicMax( &I.candKey, key );
		}
	}
}

__global__ void k_isl_sleep_flags( DIslands* Ip )
{
	DIslands& I = *Ip;
	int n = I.awakeIslandCount;
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
		I.flag[i] = I.islandBits[i] ? 0 : 1;
}

// Keep-awake bits and the split candidate in awake order (solver.c:658-675),
// then islands whose bit stayed clear fall asleep, last first
// (solver.c:2003-2048).
__global__ void k_isl_sleep( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	if ( I.moveCount == 0 || w.enableSleep == 0 )
		return;
	int candidate = ISL_NULL;
	if ( I.candKey != 0ull )
	{
		int i = (int)( 0xffffffffu - (unsigned)( I.candKey & 0xffffffffull ) );
		candidate = I.bIsland[I.awakeBodies[i]];
	}
	I.splitIslandId = candidate;
	// islands whose bit stayed clear, listed in array order: last first
	for ( int k = I.listCount - 1; k >= 0; --k )
		isl_try_sleep( w, I, I.list[k] );
}

// b2Body_SetAwake (body.c:1483-1508), b2Body_EnableSleep(false) and the wake
// of b2Body_Apply*/SetVelocity (wake = 1), b2World_EnableSleeping(false)
// (world.c:1710-1740): op 0 wake the body's set, 1 put its island to sleep,
// 2 wake every sleeping set.
__global__ void k_isl_api( DWorld w, DIslands* Ip, int op, int body )
{
	DIslands& I = *Ip;
	if ( op == 0 )
	{
		if ( I.bSet[body] >= SET_FIRST_SLEEPING )
			isl_wake_set( w, I, I.bSet[body] );
	}
	else if ( op == 1 )
	{
		if ( I.bSet[body] == SET_AWAKE )
		{
			if ( I.islands[I.bIsland[body]].removeCount > 0 )
				isl_split( w, I, I.bIsland[body] );
			isl_try_sleep( w, I, I.bIsland[body] );
		}
	}
	else
	{
		for ( int s = SET_FIRST_SLEEPING; s < I.setNext; ++s )
			if ( I.sets[s].used && I.sets[s].bodyCount > 0 )
				isl_wake_set( w, I, s );
	}
}

// Wakes the sleeping sets of the blast's shapes' bodies in the order the
// reference's query visits them (b2WakeBody per blast shape, world.c:2673):
// byRank[r] is the shape at left-to-right tree position r (or -1), visited
// from the last position down.
__global__ void k_isl_wake_marked( DWorld w, DIslands* Ip, const int* byRank, int n )
{
	DIslands& I = *Ip;
	for ( int r = n - 1; r >= 0; --r )
	{
		int s = byRank[r];
		if ( s < 0 || s >= w.shapeCount )
			continue;
		int b = w.shapeBody[s];
		if ( I.bSet[b] >= SET_FIRST_SLEEPING )
			isl_wake_set( w, I, I.bSet[b] );
	}
}

// Solver set per body for the state dump (0 static, 1 disabled, 2 awake, 3..).
__global__ void k_isl_body_sets( DWorld w, DIslands* Ip, int* out, int n )
{
	for ( int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x )
		out[b] = Ip->bSet[b];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void launch_isl_create( DWorld& w, cudaStream_t st )
{
	k_isl_create<<<1, 1, 0, st>>>( w, w.isl );
}

// Native order in parallel: the new contacts are the first newPairCount ids
// the pool hands out (LIFO free ids, then fresh ones), those created in
// creation order; their set records start in parallel and their body edges,
// sorted by (body, creation rank), are prepended in rank order per body --
// the list the serial prepends (contact.c:227-262) give.
__global__ void k_isl_nc_flags( DWorld w, int* ids, int* flag )
{
	int n = min( w.sc->newPairCount, w.pairCap );
	int F = w.sc->contactFreeCount;
	int base = w.sc->contactIdCount;
	for ( int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x )
	{
		int id = r < F ? w.contactFree[F - 1 - r] : base + ( r - F );
		bool ok = id >= 0 && id < w.contactCap && ( w.cflags[id] & CF_USED ) != 0;
		ids[r] = id;
		flag[r] = ok ? 1 : 0;
	}
}

__global__ void k_isl_nc_init( DWorld w, DIslands* Ip, const int* ids, const int* flag, const int* pos )
{
	DIslands& I = *Ip;
	int n = min( w.sc->newPairCount, w.pairCap );
	for ( int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x )
	{
		if ( !flag[r] )
			continue;
		int i = pos[r];
		int c = ids[r];
		I.order[i] = c;
		int2 bd = w.cbody[c];
		bool awake = I.bSet[bd.x] == SET_AWAKE || I.bSet[bd.y] == SET_AWAKE;
		I.cSet[c] = awake ? SET_AWAKE : SET_DISABLED;
		I.cIsland[c] = I.cIslandPrev[c] = I.cIslandNext[c] = ISL_NULL;
		I.cMark[c] = 0;
		if ( !awake )
			w.cflags[c] |= CF_INACTIVE;
		I.ncKeys[2 * i] = ( (unsigned long long)(unsigned)bd.x << 32 ) | (unsigned)( 2 * i );
		I.ncKeys[2 * i + 1] = ( (unsigned long long)(unsigned)bd.y << 32 ) | (unsigned)( 2 * i + 1 );
	}
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
		I.ncCount = 2 * ( n > 0 ? pos[n - 1] + flag[n - 1] : 0 );
}

// edge key of sorted row p: (contact << 1) | edge
__device__ __forceinline__ int nc_edge_key( const DIslands& I, unsigned long long k )
{
	int idx = (int)( k & 0xffffffffull );
	return ( I.order[idx >> 1] << 1 ) | ( idx & 1 );
}

__global__ void k_isl_nc_chain( DIslands* Ip )
{
	DIslands& I = *Ip;
	int n = I.ncCount;
	for ( int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x )
	{
		unsigned long long k = I.ncKeys[p];
		unsigned b = (unsigned)( k >> 32 );
		int key = nc_edge_key( I, k );
		bool first = p == 0 || (unsigned)( I.ncKeys[p - 1] >> 32 ) != b;
		bool last = p + 1 == n || (unsigned)( I.ncKeys[p + 1] >> 32 ) != b;
		int next, prev = last ? ISL_NULL : nc_edge_key( I, I.ncKeys[p + 1] );
		if ( first )
		{
			next = I.bHeadContact[b];
			if ( next != ISL_NULL )
				( (int*)( I.cEdge + ( next >> 1 ) ) )[( next & 1 ) ? 2 : 0] = key;
		}
		else
			next = nc_edge_key( I, I.ncKeys[p - 1] );
		int* e = (int*)( I.cEdge + ( key >> 1 ) );
		e[( key & 1 ) ? 3 : 1] = next;
		e[( key & 1 ) ? 2 : 0] = prev;
	}
}

__global__ void k_isl_nc_heads( DIslands* Ip )
{
	DIslands& I = *Ip;
	int n = I.ncCount;
	for ( int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x )
	{
		unsigned long long k = I.ncKeys[p];
		unsigned b = (unsigned)( k >> 32 );
		if ( p + 1 == n || (unsigned)( I.ncKeys[p + 1] >> 32 ) != b )
			I.bHeadContact[b] = nc_edge_key( I, k );
	}
}

void launch_isl_new_contacts( DWorld& w, StepScratch& s, cudaStream_t st, int planMode )
{
	if ( planMode )
	{
		k_isl_new_contacts<<<1, 1, 0, st>>>( w, w.isl, planMode );
		return;
	}
	DIslands* I = w.isl;
	int* ids = s.tmpA;
	int* flag = s.tmpA + w.pairCap;
	int* pos = s.tmpB;
	int g = grid_for( w.pairCap );
	k_isl_nc_flags<<<g, 256, 0, st>>>( w, ids, flag );
	scan_lookback( flag, pos, &w.sc->newPairCount, 0, w.pairCap, nullptr, s.scanState, &w.sc->error, st );
	k_isl_nc_init<<<g, 256, 0, st>>>( w, I, ids, flag, pos );
	int bodyBits = 1;
	while ( ( 1 << bodyBits ) < w.bodyCap )
		bodyBits += 1;
	int* count = (int*)( (char*)I + offsetof( DIslands, ncCount ) );
	unsigned long long* k0 = w.islNcKeys;
	unsigned long long* k1 = w.islNcKeysAlt;
	sort_coop<unsigned long long>( k0, nullptr, k1, nullptr, count, 32 + bodyBits, w.sortHist, &w.sc->barrierCount,
								   &w.sc->error, s.sortBlocks64, st );
	int g2 = grid_for( 2 * w.pairCap );
	k_isl_nc_chain<<<g2, 256, 0, st>>>( I );
	k_isl_nc_heads<<<g2, 256, 0, st>>>( I );
}

static int* isl_field( DIslands* I, size_t offset )
{
	return (int*)( (char*)I + offset );
}

static void isl_list( DWorld& w, unsigned long long* scanState, cudaStream_t st )
{
	int* count = isl_field( w.isl, offsetof( DIslands, awakeIslandCount ) );
	int* total = isl_field( w.isl, offsetof( DIslands, listCount ) );
	scan_lookback( w.islFlag, w.islPos, count, 0, w.bodyCap, total, scanState, &w.sc->error, st );
	k_isl_list<<<grid_for( w.bodyCap ), 256, 0, st>>>( w.isl, count );
}

// parallel form, step 1: mark the contacts that leave an island list (end
// of touching, destroy) and the body edge lists (destroy)
__global__ void k_isl_unlink_mark( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	int nOps = min( w.sc->opCount, w.opCap );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		int kind = w.opKind[k];
		if ( kind == 1 )
			continue;
		int c = w.opContact[k];
		int m = ( I.cIsland[c] != ISL_NULL ? 1 : 0 ) | ( kind == 0 ? 2 : 0 );
		I.cRemoved[c] = (unsigned char)m;
	}
}

// step 2: every maximal run of marked nodes is cut out by the thread of its
// first node (the one whose predecessor stays): predecessor and successor
// are joined, or the list's head / tail moves. Each boundary field has one
// writer; the marked nodes keep their links until step 3.
__global__ void k_isl_unlink_runs( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	int nOps = min( w.sc->opCount, w.opCap );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		int kind = w.opKind[k];
		if ( kind == 1 )
			continue;
		int c = w.opContact[k];
		int m = I.cRemoved[c];
		if ( m & 1 )
		{
			int prev = I.cIslandPrev[c];
			if ( prev == ISL_NULL || ( I.cRemoved[prev] & 1 ) == 0 )
			{
				int next = I.cIslandNext[c];
				for ( int g = 0; next != ISL_NULL && ( I.cRemoved[next] & 1 ) && g < I.contactCap; ++g )
					next = I.cIslandNext[next];
				DIsland& isl = I.islands[I.cIsland[c]];
				if ( prev != ISL_NULL )
					I.cIslandNext[prev] = next;
				else
					isl.headContact = next;
				if ( next != ISL_NULL )
					I.cIslandPrev[next] = prev;
				else
					isl.tailContact = prev;
			}
		}
		if ( m & 2 )
		{
			int2 bd = w.cbody[c];
			for ( int edge = 0; edge < 2; ++edge )
			{
				int4 e = I.cEdge[c];
				int prev = edge == 0 ? e.x : e.z;
				if ( prev != ISL_NULL && ( I.cRemoved[prev >> 1] & 2 ) )
					continue;
				int next = edge == 0 ? e.y : e.w;
				for ( int g = 0; next != ISL_NULL && ( I.cRemoved[next >> 1] & 2 ) && g < 2 * I.contactCap; ++g )
				{
					int4 ne = I.cEdge[next >> 1];
					next = ( next & 1 ) ? ne.w : ne.y;
				}
				if ( prev != ISL_NULL )
					( (int*)( I.cEdge + ( prev >> 1 ) ) )[( prev & 1 ) ? 3 : 1] = next;
				else
					I.bHeadContact[edge == 0 ? bd.x : bd.y] = next;
				if ( next != ISL_NULL )
					( (int*)( I.cEdge + ( next >> 1 ) ) )[( next & 1 ) ? 2 : 0] = prev;
			}
		}
	}
}

// step 3: the marked nodes leave (island counts: island.c:221-261)
__global__ void k_isl_unlink_clear( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	int nOps = min( w.sc->opCount, w.opCap );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		if ( w.opKind[k] == 1 )
			continue;
		int c = w.opContact[k];
		int m = I.cRemoved[c];
		if ( m & 1 )
		{
			DIsland* isl = I.islands + I.cIsland[c];
			atomicSub( &isl->contactCount, 1 );
			atomicAdd( &isl->removeCount, 1 );
			I.cIsland[c] = I.cIslandPrev[c] = I.cIslandNext[c] = ISL_NULL;
		}
		if ( m & 2 )
			I.cEdge[c] = make_int4( ISL_NULL, ISL_NULL, ISL_NULL, ISL_NULL );
		I.cRemoved[c] = 0;
	}
}

// step 4: links of the contacts that began touching (island.c:116-219). The
// island a link prepends to is the body's island when both bodies share one
// (decided in parallel), else the union-find root at that point of the op
// order, which a serial pass over those ops alone finds (making the B root a
// child of the A root as it goes). The prepends themselves then run in
// parallel: sorted by (island, op), each island's new contacts chain in op
// order in front of its old head.
__global__ void k_isl_link_flags( DWorld w, DIslands* Ip, int* flag )
{
	const DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	int nOps = min( w.sc->opCount, w.opCap );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		int target = ISL_NULL;
		bool link = w.opKind[k] == 1;
		if ( link )
		{
			int2 bd = w.cbody[w.opContact[k]];
			int idA = I.bIsland[bd.x], idB = I.bIsland[bd.y];
			if ( idA == idB )
				target = idA;
		}
		I.order[k] = target;
		flag[k] = link ? 1 : 0;
	}
}

// The unions of the links between two islands, in op order (island.c:251-
// 289: the root choice depends on it). One block: its threads read 1024 ops
// and their bodies' islands at once and list the ones that link two
// islands in op order (warp ballots, then the warps' offsets); thread 0
// then walks their roots one after another.
#define LINK_ROOTS_THREADS 1024
__global__ void __launch_bounds__( LINK_ROOTS_THREADS ) k_isl_link_roots( DWorld w, DIslands* Ip )
{
	__shared__ int sK[LINK_ROOTS_THREADS], sA[LINK_ROOTS_THREADS], sB[LINK_ROOTS_THREADS];
	__shared__ int sWarp[LINK_ROOTS_THREADS / 32 + 1];
	DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
	int nOps = min( w.sc->opCount, w.opCap );
	for ( int base = 0; base < nOps; base += LINK_ROOTS_THREADS )
	{
		int k = base + tid;
		bool need = false;
		int idA = ISL_NULL, idB = ISL_NULL;
		if ( k < nOps && w.opKind[k] == 1 && I.order[k] == ISL_NULL )
		{
			int2 bd = w.cbody[w.opContact[k]];
			idA = I.bIsland[bd.x];
			idB = I.bIsland[bd.y];
			need = true;
		}
		unsigned m = __ballot_sync( 0xffffffffu, need );
		if ( lane == 0 )
			sWarp[wid] = __popc( m );
		__syncthreads();
		if ( tid == 0 )
		{
			int total = 0;
			for ( int i = 0; i < LINK_ROOTS_THREADS / 32; ++i )
			{
				int c = sWarp[i];
				sWarp[i] = total;
				total += c;
			}
			sWarp[LINK_ROOTS_THREADS / 32] = total;
		}
		__syncthreads();
		if ( need )
		{
			int pos = sWarp[wid] + __popc( m & ( ( 1u << lane ) - 1u ) );
			sK[pos] = k;
			sA[pos] = idA;
			sB[pos] = idB;
		}
		__syncthreads();
		if ( tid == 0 )
		{
			int cnt = sWarp[LINK_ROOTS_THREADS / 32];
			for ( int i = 0; i < cnt; ++i )
			{
				int a = sA[i], b = sB[i];
				int rootA = a != ISL_NULL ? isl_root( I, a ) : ISL_NULL;
				int rootB = b != ISL_NULL ? isl_root( I, b ) : ISL_NULL;
				if ( rootA != rootB && rootA != ISL_NULL && rootB != ISL_NULL )
					I.islands[rootB].parent = rootA;
				I.order[sK[i]] = rootA != ISL_NULL ? rootA : rootB;
			}
		}
		__syncthreads();
	}
}

__global__ void k_isl_link_keys( DWorld w, DIslands* Ip, const int* flag, const int* pos )
{
	DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	int nOps = min( w.sc->opCount, w.opCap );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		if ( !flag[k] )
			continue;
		int c = w.opContact[k];
		w.cflags[c] |= CF_TOUCHING;
		I.ncKeys[pos[k]] = ( (unsigned long long)(unsigned)I.order[k] << 32 ) | (unsigned)k;
	}
	if ( blockIdx.x == 0 && threadIdx.x == 0 )
		Ip->linkCount = nOps > 0 ? pos[nOps - 1] + flag[nOps - 1] : 0;
}

__global__ void k_isl_link_chain( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	int n = I.linkCount;
	for ( int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x )
	{
		unsigned long long key = I.ncKeys[p];
		int id = (int)( key >> 32 );
		int c = w.opContact[(int)( key & 0xffffffffull )];
		bool first = p == 0 || (int)( I.ncKeys[p - 1] >> 32 ) != id;
		bool last = p + 1 == n || (int)( I.ncKeys[p + 1] >> 32 ) != id;
		DIsland& isl = I.islands[id];
		int next;
		if ( first )
			I.pos[id] = p; // the segment's first position, for k_isl_link_heads
		if ( first )
		{
			// the island's old head and tail (written below only by the
			// segment's last / first thread, after these reads by the same
			// or an earlier thread of the segment: read them here)
			next = isl.headContact;
			if ( next != ISL_NULL )
				I.cIslandPrev[next] = c;
		}
		else
			next = w.opContact[(int)( I.ncKeys[p - 1] & 0xffffffffull )];
		I.cIslandNext[c] = next;
		I.cIslandPrev[c] = last ? ISL_NULL : w.opContact[(int)( I.ncKeys[p + 1] & 0xffffffffull )];
		I.cIsland[c] = id;
	}
}

// heads, tails and counts of the islands that gained contacts
__global__ void k_isl_link_heads( DWorld w, DIslands* Ip )
{
	DIslands& I = *Ip;
	if ( I.serialOps )
		return;
	int n = I.linkCount;
	for ( int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x )
	{
		unsigned long long key = I.ncKeys[p];
		int id = (int)( key >> 32 );
		bool last = p + 1 == n || (int)( I.ncKeys[p + 1] >> 32 ) != id;
		if ( !last )
			continue;
		int q = I.pos[id];
		DIsland& isl = I.islands[id];
		int c = w.opContact[(int)( key & 0xffffffffull )];
		if ( isl.tailContact == ISL_NULL )
			isl.tailContact = w.opContact[(int)( I.ncKeys[q] & 0xffffffffull )];
		isl.headContact = c;
		isl.contactCount += p - q + 1;
	}
}

void launch_isl_ops( DWorld& w, StepScratch& s, cudaStream_t st, const int* gkind )
{
	unsigned long long* scanState = s.scanState;
	int g = grid_for( w.opCap );
	cudaMemsetAsync( (char*)w.isl + offsetof( DIslands, serialOps ), 0, sizeof( int ), st );
	k_isl_op_check<<<g, 256, 0, st>>>( w, w.isl );
	k_isl_ops<<<1, 1, 0, st>>>( w, w.isl, gkind );
	k_isl_unlink_mark<<<g, 256, 0, st>>>( w, w.isl );
	k_isl_unlink_runs<<<g, 256, 0, st>>>( w, w.isl );
	k_isl_unlink_clear<<<g, 256, 0, st>>>( w, w.isl );
	// links: flags and same-island targets, the serial unions, then the
	// prepends sorted by (island, op) (scratch past the op kinds in tmpA)
	int* flag = s.tmpA + w.opCap;
	int* pos = s.tmpB;
	k_isl_link_flags<<<g, 256, 0, st>>>( w, w.isl, flag );
	k_isl_link_roots<<<1, LINK_ROOTS_THREADS, 0, st>>>( w, w.isl );
	scan_lookback( flag, pos, &w.sc->opCount, 0, w.opCap, nullptr, scanState, &w.sc->error, st );
	k_isl_link_keys<<<g, 256, 0, st>>>( w, w.isl, flag, pos );
	int islandBits = 1;
	while ( ( 1 << islandBits ) < w.bodyCap + 1 )
		islandBits += 1;
	sort_coop<unsigned long long>( w.islNcKeys, nullptr, w.islNcKeysAlt, nullptr,
								   (int*)( (char*)w.isl + offsetof( DIslands, linkCount ) ), 32 + islandBits, w.sortHist,
								   &w.sc->barrierCount, &w.sc->error, s.sortBlocks64, st );
	k_isl_link_chain<<<g, 256, 0, st>>>( w, w.isl );
	k_isl_link_heads<<<g, 256, 0, st>>>( w, w.isl );
	k_isl_merge_roots<<<grid_for( w.bodyCap ), 256, 0, st>>>( w, w.isl );
	isl_list( w, scanState, st );
	k_isl_merge_remap<<<grid_for( w.bodyCap + w.contactCap + w.jointCap ), 256, 0, st>>>( w, w.isl );
	k_isl_merge_apply<<<1, 1, 0, st>>>( w.isl );
}

void launch_isl_split( DWorld& w, cudaStream_t st )
{
	k_isl_split<<<1, 1, 0, st>>>( w, w.isl );
	k_isl_move_slots<<<grid_for( w.bodyCap ), 256, 0, st>>>( w.isl );
}

void launch_isl_sleep( DWorld& w, cudaStream_t st, unsigned long long* scanState )
{
	k_isl_bits<<<grid_for( w.bodyCap ), 256, 0, st>>>( w, w.isl );
	k_isl_sleep_flags<<<grid_for( w.bodyCap ), 256, 0, st>>>( w.isl );
	isl_list( w, scanState, st );
	k_isl_sleep<<<1, 1, 0, st>>>( w, w.isl );
}

void launch_isl_api( DWorld& w, cudaStream_t st, int op, int body )
{
	k_isl_api<<<1, 1, 0, st>>>( w, w.isl, op, body );
}

void launch_isl_wake_marked( DWorld& w, cudaStream_t st, const int* shapeMarks, int shapeCount )
{
	k_isl_wake_marked<<<1, 1, 0, st>>>( w, w.isl, shapeMarks, shapeCount );
}

void launch_isl_body_sets( DWorld& w, cudaStream_t st, int* out, int n )
{
	k_isl_body_sets<<<grid_for( n ), 256, 0, st>>>( w, w.isl, out, n );
}

// Re-applies BF_ASLEEP to bodies whose host rows were uploaded (the host
// mirror does not track sleeping).
__global__ void k_isl_fix_flags( DWorld w, DIslands* Ip, int n )
{
	const DIslands& I = *Ip;
	int known = n < I.bodyKnown ? n : I.bodyKnown;
	for ( int b = blockIdx.x * blockDim.x + threadIdx.x; b < known; b += gridDim.x * blockDim.x )
	{
		int f = w.bflags[b];
		int s = I.bSet[b];
		w.bflags[b] = s >= SET_FIRST_SLEEPING ? ( f | BF_ASLEEP ) : ( f & ~BF_ASLEEP );
	}
}

void launch_isl_fix_flags( DWorld& w, cudaStream_t st, int n )
{
	k_isl_fix_flags<<<grid_for( n ), 256, 0, st>>>( w, w.isl, n );
}

// ---------------------------------------------------------------------------
// Destroy path, serial (between steps; one thread, the reference's order):
// contact.c:337-453 b2DestroyContact, joint.c:702-806
// b2DestroyJointInternal, body.c:99-157 b2RemoveBodyFromIsland, :412-432
// (the body leaves its solver set), island.c:58-84, :384-424. Worlds without
// sleeping keep no island records (Ip null): contacts and joints then only
// leave the constraint graph.
// ---------------------------------------------------------------------------
// The reference's set arrays lose an element by moving their last element
// into the hole; a sleeping set here is a singly linked list in array order,
// so the same move is made on the list.
template <typename Next>
__device__ void isl_list_swap_remove( int& head, int& tail, int& count, Next next, int x )
{
	bool found = false;
	int prevX = ISL_NULL, prevT = ISL_NULL;
	for ( int k = head, p = ISL_NULL, g = 0; k != ISL_NULL && g < ( 1 << 26 ); p = k, k = next( k ), ++g )
	{
		if ( k == x )
		{
			found = true;
			prevX = p;
		}
		if ( k == tail )
			prevT = p;
	}
	if ( !found )
		return;
	count -= 1;
	int t = tail;
	if ( x == t )
	{
		if ( prevX == ISL_NULL )
			head = ISL_NULL;
		else
			next( prevX ) = ISL_NULL;
		tail = prevX;
		return;
	}
	if ( prevT == x )
	{
		// x, then the last element: x simply leaves
		if ( prevX == ISL_NULL )
			head = t;
		else
			next( prevX ) = t;
		return;
	}
	next( prevT ) = ISL_NULL;
	tail = prevT;
	next( t ) = next( x );
	if ( prevX == ISL_NULL )
		head = t;
	else
		next( prevX ) = t;
}

// island.c:58-84 for an island of any set
__device__ void isl_island_destroy_any( DIslands& I, int id )
{
	int setId = I.islands[id].setIndex;
	if ( setId == SET_AWAKE )
	{
		isl_island_destroy( I, id );
		return;
	}
	if ( I.splitIslandId == id )
		I.splitIslandId = ISL_NULL;
	if ( setId >= SET_FIRST_SLEEPING )
	{
		DSet& s = I.sets[setId];
		int moved = s.tailIsland;
		isl_list_swap_remove( s.headIsland, s.tailIsland, s.islandCount,
							  [&]( int k ) -> int& { return I.islands[k].setNext; }, id );
		if ( moved != id && moved != ISL_NULL )
			I.islands[moved].localIndex = I.islands[id].localIndex;
	}
	I.islands[id].setIndex = ISL_NULL;
	I.islands[id].localIndex = ISL_NULL;
	I.islandFree[I.islandFreeCount++] = id;
}

// island.c:384-424 b2UnlinkJoint
__device__ void isl_unlink_joint( DIslands& I, int j )
{
	int id = I.jIsland[j];
	if ( id == ISL_NULL )
		return;
	DIsland& isl = I.islands[id];
	int prev = I.jIslandPrev[j], next = I.jIslandNext[j];
	if ( prev != ISL_NULL )
		I.jIslandNext[prev] = next;
	if ( next != ISL_NULL )
		I.jIslandPrev[next] = prev;
	if ( isl.headJoint == j )
		isl.headJoint = next;
	if ( isl.tailJoint == j )
		isl.tailJoint = prev;
	isl.jointCount -= 1;
	isl.removeCount += 1;
	I.jIsland[j] = I.jIslandPrev[j] = I.jIslandNext[j] = ISL_NULL;
}

// body.c:331-340 b2WakeBody
__device__ void isl_wake_body( const DWorld& w, DIslands& I, int b )
{
	if ( I.bSet[b] >= SET_FIRST_SLEEPING )
		isl_wake_set( w, I, I.bSet[b] );
}

// constraint_graph.c:290-318 without island records: the overflow index of
// a joint is its position in the overflow array
__device__ void plain_graph_remove_joint( const DWorld& w, int j )
{
	int color = w.jcolor[j];
	if ( color == F2D_NULL )
		return;
	int2 jb = w.jbody[j];
	if ( color != F2D_OVERFLOW )
	{
		// the bits its colouring set (the reference clears both bodies'
		// bits, constraint_graph.c:303-308, which differs only for a body
		// that was static when the joint was coloured and is not any more)
		unsigned bit = 1u << color;
		int set = w.jcolorSet[j];
		if ( set & 1 )
			w.colorMask[jb.x] &= ~bit;
		if ( set & 2 )
			w.colorMask[jb.y] &= ~bit;
	}
	else
	{
		int last = w.sc->overflowJointCount - 1;
		for ( int idx = 0; idx <= last; ++idx )
			if ( w.overflowJoints[idx] == j )
			{
				w.overflowJoints[idx] = w.overflowJoints[last];
				w.sc->overflowJointCount = last;
				break;
			}
	}
	w.jcolor[j] = F2D_NULL;
}

// contact.c:337-453; the end event of a touching contact with events goes to
// the destroy buffer (reported with the next step's end events)
__device__ void dev_destroy_contact( const DWorld& w, DIslands* Ip, int c, bool wake )
{
	int f = w.cflags[c];
	if ( ( f & CF_USED ) == 0 )
		return;
	bool touching = ( f & CF_TOUCHING ) != 0;
	if ( touching && ( f & CF_EVENTS ) )
	{
		int e = w.sc->apiEndCount++;
		if ( e < w.contactCap )
		{
			int2 sh = w.cshape[c];
			w.apiEndEv[2 * e] = sh.x;
			w.apiEndEv[2 * e + 1] = sh.y;
		}
	}
	int2 bd = w.cbody[c];
	if ( Ip )
	{
		DIslands& I = *Ip;
		isl_edges_unlink( w, I, c );
		isl_unlink_contact( I, c );
		if ( w.ccolor[c] != F2D_NULL )
			isl_graph_remove_contact( w, c );
		else
		{
			int s = I.cSet[c];
			if ( s >= SET_FIRST_SLEEPING )
				isl_list_swap_remove( I.sets[s].headContact, I.sets[s].tailContact, I.sets[s].contactCount,
									  [&]( int k ) -> int& { return I.cSetNext[k]; }, c );
		}
		I.cSet[c] = ISL_NULL;
	}
	else if ( w.ccolor[c] != F2D_NULL )
		isl_graph_remove_contact( w, c );
	w.cflags[c] = 0;
	w.ccolor[c] = F2D_NULL;
	w.contactFree[w.sc->contactFreeCount++] = c;
	if ( Ip && wake && touching )
	{
		isl_wake_body( w, *Ip, bd.x );
		isl_wake_body( w, *Ip, bd.y );
	}
}

// Contacts of body b in the order of its contact list (newest first): the
// island records keep the list; without them the collected contacts are
// ordered by creation stamp. Filters: only contacts with shape `shape`
// (>= 0), or only those whose other body is `other` (>= 0).
__global__ void k_collect_body_contacts( DWorld w, int b, int* out )
{
	int n = w.sc->contactIdCount;
	for ( int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x )
	{
		if ( ( w.cflags[c] & CF_USED ) == 0 )
			continue;
		int2 bd = w.cbody[c];
		if ( bd.x == b || bd.y == b )
		{
			int k = atomicAdd( &w.sc->apiCount, 1 );
			if ( k < w.contactCap )
				out[k] = c;
		}
	}
}

__global__ void k_destroy_body_contacts( DWorld w, DIslands* Ip, int b, int shape, int other, int wake, int* list )
{
	int n = 0;
	if ( Ip )
	{
		DIslands& I = *Ip;
		for ( int key = I.bHeadContact[b], g = 0; key != ISL_NULL && g < I.contactCap; ++g )
		{
			int c = key >> 1;
			int4 e = I.cEdge[c];
			list[n++] = c;
			key = ( key & 1 ) ? e.w : e.y;
		}
	}
	else
	{
		n = min( w.sc->apiCount, w.contactCap );
		// newest first
		for ( int i = 1; i < n; ++i )
		{
			int v = list[i];
			unsigned long long sv = w.cstamp[v];
			int j = i - 1;
			while ( j >= 0 && w.cstamp[list[j]] < sv )
			{
				list[j + 1] = list[j];
				j -= 1;
			}
			list[j + 1] = v;
		}
	}
	for ( int i = 0; i < n; ++i )
	{
		int c = list[i];
		int2 sh = w.cshape[c];
		int2 bd = w.cbody[c];
		if ( shape >= 0 && sh.x != shape && sh.y != shape )
			continue;
		if ( other >= 0 && ( bd.x == b ? bd.y : bd.x ) != other )
			continue;
		dev_destroy_contact( w, Ip, c, wake != 0 );
	}
	w.sc->apiCount = 0;
}

// joint.c:702-806 on the device records (the body joint lists live on the
// host and are uploaded with the body rows)
__global__ void k_destroy_joint( DWorld w, DIslands* Ip, int j, int wake )
{
	int2 jb = w.jbody[j];
	if ( Ip )
	{
		DIslands& I = *Ip;
		isl_unlink_joint( I, j );
		int s = I.jSet[j];
		if ( s == SET_AWAKE )
			isl_graph_remove_joint( w, I, j );
		else if ( s >= SET_FIRST_SLEEPING )
			isl_list_swap_remove( I.sets[s].headJoint, I.sets[s].tailJoint, I.sets[s].jointCount,
								  [&]( int k ) -> int& { return I.jSetNext[k]; }, j );
		I.jSet[j] = ISL_NULL;
	}
	else
		plain_graph_remove_joint( w, j );
	w.jflags[j] = 0;
	w.jimp[j] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	w.jimp2[j] = make_float2( 0.0f, 0.0f );
	if ( Ip && wake )
	{
		isl_wake_body( w, *Ip, jb.x );
		isl_wake_body( w, *Ip, jb.y );
	}
}

// body.c:99-157 b2RemoveBodyFromIsland: an island left without bodies goes
__device__ void isl_remove_body_from_island( DIslands& I, int b )
{
	int id = I.bIsland[b];
	if ( id == ISL_NULL )
		return;
	DIsland& isl = I.islands[id];
	int prev = I.bIslandPrev[b], next = I.bIslandNext[b];
	if ( prev != ISL_NULL )
		I.bIslandNext[prev] = next;
	if ( next != ISL_NULL )
		I.bIslandPrev[next] = prev;
	isl.bodyCount -= 1;
	if ( isl.headBody == b )
	{
		isl.headBody = next;
		if ( next == ISL_NULL )
			isl_island_destroy_any( I, id );
	}
	else if ( isl.tailBody == b )
		isl.tailBody = prev;
	I.bIsland[b] = I.bIslandPrev[b] = I.bIslandNext[b] = ISL_NULL;
}

// body.c:84-96 b2CreateIslandForBody
__device__ void isl_create_island_for_body( DIslands& I, int setId, int b )
{
	int isl = isl_island_create( I, setId );
	I.bIsland[b] = isl;
	I.bIslandPrev[b] = I.bIslandNext[b] = ISL_NULL;
	I.islands[isl].headBody = I.islands[isl].tailBody = b;
	I.islands[isl].bodyCount = 1;
}

// body.c:99-157 and :412-432: out of its island and its solver set
__global__ void k_destroy_body_records( DWorld w, DIslands* Ip, int b )
{
	if ( Ip )
	{
		DIslands& I = *Ip;
		isl_remove_body_from_island( I, b );
		int s = I.bSet[b];
		if ( s == SET_AWAKE )
			isl_awake_remove_body( I, b );
		else if ( s >= SET_FIRST_SLEEPING )
		{
			DSet& set = I.sets[s];
			isl_list_swap_remove( set.headBody, set.tailBody, set.bodyCount,
								  [&]( int k ) -> int& { return I.bSetNext[k]; }, b );
			if ( set.bodyCount == 0 )
				isl_set_destroy( I, s );
		}
		I.bSet[b] = ISL_NULL;
		I.bHeadContact[b] = ISL_NULL;
	}
	w.bflags[b] = 0;
}

// ---------------------------------------------------------------------------
// type changes, disable and enable (body.c:1036-1282, 1557-1700) on the
// device records, one thread; the host destroys the body's contacts before
// (launch_destroy_contacts_of) and re-creates its proxies after. Worlds
// without islands keep no set records: there a joint is in the awake set
// when it holds a colour, in the disabled set when a body is disabled and in
// the static set otherwise.
// ---------------------------------------------------------------------------
__device__ int joint_set_of( const DWorld& w, DIslands* Ip, int j )
{
	if ( Ip )
		return Ip->jSet[j];
	if ( w.jcolor[j] != F2D_NULL )
		return SET_AWAKE;
	int2 jb = w.jbody[j];
	if ( ( w.bflags[jb.x] & BF_ENABLED ) == 0 || ( w.bflags[jb.y] & BF_ENABLED ) == 0 )
		return SET_DISABLED;
	return SET_STATIC;
}

// k_joint_ops' colouring for a world without islands (overflow joints keep
// no index there)
__device__ void plain_graph_add_joint( const DWorld& w, int j )
{
	int2 jb = w.jbody[j];
	int a = isl_static( w, jb.x ) ? -1 : jb.x, b = isl_static( w, jb.y ) ? -1 : jb.y;
	int color = F2D_OVERFLOW;
	for ( int c = 0; c < F2D_OVERFLOW && ( a >= 0 || b >= 0 ); ++c )
	{
		unsigned used = ( a >= 0 ? w.colorMask[a] : 0u ) | ( b >= 0 ? w.colorMask[b] : 0u );
		if ( ( used & ( 1u << c ) ) == 0 )
		{
			color = c;
			break;
		}
	}
	if ( color != F2D_OVERFLOW )
	{
		if ( a >= 0 )
			w.colorMask[a] |= 1u << color;
		if ( b >= 0 )
			w.colorMask[b] |= 1u << color;
	}
	w.jcolor[j] = color;
	w.jcolorSet[j] = color == F2D_OVERFLOW ? 0 : ( a >= 0 ? 1 : 0 ) | ( b >= 0 ? 2 : 0 );
	if ( color == F2D_OVERFLOW )
	{
		w.overflowJoints[w.sc->overflowJointCount] = j;
		w.sc->overflowJointCount += 1;
	}
}

// solver_set.c:558-613 b2TransferJoint: out of the graph (awake) or the
// source set's list, into the graph (awake) or the target set's list
__device__ void transfer_joint( const DWorld& w, DIslands* Ip, int j, int target )
{
	int src = joint_set_of( w, Ip, j );
	if ( src == SET_AWAKE )
	{
		if ( Ip )
			isl_graph_remove_joint( w, *Ip, j );
		else
			plain_graph_remove_joint( w, j );
	}
	else if ( Ip && src >= SET_FIRST_SLEEPING )
		isl_list_swap_remove( Ip->sets[src].headJoint, Ip->sets[src].tailJoint, Ip->sets[src].jointCount,
							  [&]( int k ) -> int& { return Ip->jSetNext[k]; }, j );
	if ( target == SET_AWAKE )
	{
		if ( Ip )
		{
			Ip->jSet[j] = SET_AWAKE;
			isl_graph_add_joint( w, *Ip, j );
		}
		else
			plain_graph_add_joint( w, j );
	}
	else if ( Ip && target >= SET_FIRST_SLEEPING )
		isl_set_push_joint( *Ip, target, j );
	else if ( Ip )
		Ip->jSet[j] = target;
}

// b2_identityBodyState: a body entering or leaving the awake set
__device__ void identity_state( const DWorld& w, int b )
{
	w.vel[b] = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	w.delta[b] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
}

#define JOINT_KEYS( w, b, key, j )                                                                                      \
	for ( int key = ( w ).headJoint[b], j = key >> 1, guard_ = 0; key != F2D_NULL && guard_ <= ( w ).jointCount;     \
		  key = ( w ).jnext[2 * j + ( key & 1 )], j = key >> 1, ++guard_ )

// body.c:1036-1282 b2Body_SetType
__global__ void k_body_set_type( DWorld w, DIslands* Ip, int b, int type )
{
	int orig = body_type( w.bflags[b] );
	if ( Ip )
	{
		isl_wake_body( w, *Ip, b );
		JOINT_KEYS( w, b, key, j )
		{
			int2 jb = w.jbody[j];
			if ( Ip->jIsland[j] != ISL_NULL )
				isl_unlink_joint( *Ip, j );
			isl_wake_body( w, *Ip, jb.x );
			isl_wake_body( w, *Ip, jb.y );
		}
	}
	// the joints' sets before the type changes
	w.bflags[b] = ( w.bflags[b] & ~( 3 << BF_TYPE_SHIFT ) ) | ( type << BF_TYPE_SHIFT );
	if ( orig == 0 )
	{
		if ( Ip )
		{
			isl_awake_add_body( w, *Ip, b );
			isl_create_island_for_body( *Ip, SET_AWAKE, b );
		}
		identity_state( w, b );
		JOINT_KEYS( w, b, key, j )
		{
			int s = joint_set_of( w, Ip, j );
			if ( s == SET_STATIC )
				transfer_joint( w, Ip, j, SET_AWAKE );
			else if ( s == SET_AWAKE )
			{
				// back into the graph for its colour
				transfer_joint( w, Ip, j, SET_STATIC );
				transfer_joint( w, Ip, j, SET_AWAKE );
			}
		}
	}
	else if ( type == 0 )
	{
		if ( Ip )
		{
			isl_awake_remove_body( *Ip, b );
			Ip->bSet[b] = SET_STATIC;
			isl_remove_body_from_island( *Ip, b );
		}
		identity_state( w, b );
		w.bflags[b] &= ~BF_IS_FAST;
		JOINT_KEYS( w, b, key, j )
		{
			int2 jb = w.jbody[j];
			int other = ( key & 1 ) ? jb.x : jb.y;
			int s = joint_set_of( w, Ip, j );
			if ( s == SET_DISABLED )
				continue;
			transfer_joint( w, Ip, j, SET_STATIC );
			if ( body_type( w.bflags[other] ) != 0 )
				transfer_joint( w, Ip, j, SET_AWAKE );
		}
	}
	if ( Ip )
	{
		JOINT_KEYS( w, b, key, j )
		{
			int2 jb = w.jbody[j];
			int other = ( key & 1 ) ? jb.x : jb.y;
			if ( Ip->bSet[other] == SET_DISABLED )
				continue;
			if ( type == 0 && body_type( w.bflags[other] ) == 0 )
				continue;
			isl_link_joint( w, *Ip, j, false );
		}
		isl_merge_awake( *Ip );
	}
}

// body.c:1557-1626 b2Body_Disable (contacts destroyed and proxies removed by
// the host)
__global__ void k_body_disable( DWorld w, DIslands* Ip, int b )
{
	int f = w.bflags[b];
	int src = body_type( f ) == 0 ? SET_STATIC : SET_AWAKE;
	if ( Ip )
	{
		DIslands& I = *Ip;
		isl_remove_body_from_island( I, b );
		src = I.bSet[b];
		if ( src == SET_AWAKE )
			isl_awake_remove_body( I, b );
		else if ( src >= SET_FIRST_SLEEPING )
			isl_list_swap_remove( I.sets[src].headBody, I.sets[src].tailBody, I.sets[src].bodyCount,
								  [&]( int k ) -> int& { return I.bSetNext[k]; }, b );
		I.bSet[b] = SET_DISABLED;
	}
	if ( src == SET_AWAKE )
		identity_state( w, b );
	JOINT_KEYS( w, b, key, j )
	{
		int s = joint_set_of( w, Ip, j );
		if ( s == SET_DISABLED )
			continue;
		if ( Ip && Ip->jIsland[j] != ISL_NULL )
			isl_unlink_joint( *Ip, j );
		transfer_joint( w, Ip, j, SET_DISABLED );
	}
	w.bflags[b] = f & ~BF_ENABLED;
}

// body.c:1628-1700 b2Body_Enable (proxies re-created by the host)
__global__ void k_body_enable( DWorld w, DIslands* Ip, int b )
{
	int setId = body_type( w.bflags[b] ) == 0 ? SET_STATIC : SET_AWAKE;
	w.bflags[b] |= BF_ENABLED;
	if ( Ip )
	{
		if ( setId == SET_AWAKE )
			isl_awake_add_body( w, *Ip, b );
		else
			Ip->bSet[b] = SET_STATIC;
	}
	if ( setId == SET_AWAKE )
		identity_state( w, b );
	if ( Ip && setId != SET_STATIC )
		isl_create_island_for_body( *Ip, setId, b );
	JOINT_KEYS( w, b, key, j )
	{
		int2 jb = w.jbody[j];
		if ( ( w.bflags[jb.x] & BF_ENABLED ) == 0 || ( w.bflags[jb.y] & BF_ENABLED ) == 0 )
			continue;
		bool sa = body_type( w.bflags[jb.x] ) == 0, sb = body_type( w.bflags[jb.y] ) == 0;
		int jointSet = SET_STATIC;
		if ( Ip )
		{
			int ba = Ip->bSet[jb.x], bb = Ip->bSet[jb.y];
			jointSet = ( sa && sb ) ? SET_STATIC : ( ba == SET_STATIC ? bb : ba );
			// from the disabled set
			Ip->jSet[j] = SET_DISABLED;
		}
		else if ( !( sa && sb ) )
			jointSet = SET_AWAKE;
		transfer_joint( w, Ip, j, jointSet );
		if ( Ip && jointSet != SET_STATIC )
			isl_link_joint( w, *Ip, j, false );
	}
	if ( Ip )
		isl_merge_awake( *Ip );
}

void launch_body_set_type( DWorld& w, cudaStream_t st, int body, int type )
{
	k_body_set_type<<<1, 1, 0, st>>>( w, w.isl, body, type );
}

void launch_body_disable( DWorld& w, cudaStream_t st, int body )
{
	k_body_disable<<<1, 1, 0, st>>>( w, w.isl, body );
}

void launch_body_enable( DWorld& w, cudaStream_t st, int body )
{
	k_body_enable<<<1, 1, 0, st>>>( w, w.isl, body );
}

// broad_phase.c:70-88 b2UnBufferMove: the proxy leaves the move array by
// swap-remove
__global__ void k_unbuffer_move( DWorld w, int s )
{
	int f = w.sflags[s];
	if ( ( f & SF_MOVED ) == 0 )
		return;
	int idx = w.shapeMove[s];
	int last = w.sc->moveArrayCount - 1;
	if ( idx != last )
	{
		int m = w.moveShape[last];
		w.moveShape[idx] = m;
		w.shapeMove[m] = idx;
	}
	w.sc->moveArrayCount = last;
	w.sflags[s] = f & ~SF_MOVED;
}

void launch_destroy_contacts_of( DWorld& w, cudaStream_t st, int body, int shape, int other, int wake, int* list )
{
	if ( !w.isl )
		k_collect_body_contacts<<<grid_for( w.contactCap ), 256, 0, st>>>( w, body, list );
	k_destroy_body_contacts<<<1, 1, 0, st>>>( w, w.isl, body, shape, other, wake, list );
}

void launch_destroy_joint( DWorld& w, cudaStream_t st, int joint, int wake )
{
	k_destroy_joint<<<1, 1, 0, st>>>( w, w.isl, joint, wake );
}

void launch_destroy_body_records( DWorld& w, cudaStream_t st, int body )
{
	k_destroy_body_records<<<1, 1, 0, st>>>( w, w.isl, body );
}

void launch_unbuffer_move( DWorld& w, cudaStream_t st, int shape )
{
	k_unbuffer_move<<<1, 1, 0, st>>>( w, shape );
}
