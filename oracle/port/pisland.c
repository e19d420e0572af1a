// Islands and solver sets of the CPU restatement: persistent islands
// (union on touch begin, lazy split of the sleepiest island), sleeping
// solver sets and waking, as island.c and solver_set.c do. TEST
// INFRASTRUCTURE (oracle). Set and list orders follow the reference exactly
// because they decide which contacts re-enter the constraint graph, and in
// what order, when a set wakes.
#include "port.h"

#include <stdlib.h>
#include <string.h>

// ---------------------------------------------------------------------------
// growable arrays and id pools (array.h, id_pool.c:19-38)
// ---------------------------------------------------------------------------
void ia_push( IntArr* a, int v )
{
	if ( a->count == a->cap )
	{
		int cap = a->cap < 8 ? 8 : 2 * a->cap;
		a->data = (int*)realloc( a->data, sizeof( int ) * (size_t)cap );
		a->cap = cap;
	}
	a->data[a->count++] = v;
}

// b2Array_RemoveSwap: returns the index the last element moved from, or
// P_NULL when the removed element was the last one.
int ia_remove_swap( IntArr* a, int index )
{
	int last = a->count - 1;
	if ( index != last )
	{
		a->data[index] = a->data[last];
		a->count -= 1;
		return last;
	}
	a->count -= 1;
	return P_NULL;
}

void ia_free( IntArr* a )
{
	free( a->data );
	a->data = NULL;
	a->count = a->cap = 0;
}

static int pool_alloc( IdPool* p )
{
	if ( p->freeIds.count > 0 )
		return p->freeIds.data[--p->freeIds.count];
	return p->next++;
}

static void pool_free( IdPool* p, int id )
{
	ia_push( &p->freeIds, id );
}

// ---------------------------------------------------------------------------
// solver sets (solver_set.c)
// ---------------------------------------------------------------------------
static SolverSet* set_get( World* w, int id )
{
	return w->sets + id;
}

static int set_create( World* w )
{
	int id = pool_alloc( &w->setPool );
	if ( id >= w->setCap )
	{
		int cap = w->setCap < 8 ? 8 : 2 * w->setCap;
		while ( cap <= id )
			cap *= 2;
		w->sets = (SolverSet*)realloc( w->sets, sizeof( SolverSet ) * (size_t)cap );
		memset( w->sets + w->setCap, 0, sizeof( SolverSet ) * (size_t)( cap - w->setCap ) );
		w->setCap = cap;
	}
	SolverSet* s = w->sets + id;
	s->setIndex = id;
	s->bodies.count = s->contacts.count = s->joints.count = s->islands.count = 0;
	return id;
}

static void set_destroy( World* w, int id )
{
	SolverSet* s = w->sets + id;
	s->setIndex = P_NULL;
	s->bodies.count = s->contacts.count = s->joints.count = s->islands.count = 0;
	pool_free( &w->setPool, id );
}

void p_sets_init( World* w )
{
	// world.c: the static, disabled and awake sets take ids 0, 1, 2
	for ( int k = 0; k < SET_FIRST_SLEEPING; ++k )
		set_create( w );
	w->splitIslandId = P_NULL;
}

void p_sets_free( World* w )
{
	for ( int i = 0; i < w->setCap; ++i )
	{
		ia_free( &w->sets[i].bodies );
		ia_free( &w->sets[i].contacts );
		ia_free( &w->sets[i].joints );
		ia_free( &w->sets[i].islands );
	}
	free( w->sets );
	w->sets = NULL;
	w->setCap = 0;
	ia_free( &w->setPool.freeIds );
	free( w->islands );
	w->islands = NULL;
	w->islandCap = 0;
	ia_free( &w->islandPool.freeIds );
	free( w->moveEventAsleep );
	w->moveEventAsleep = NULL;
}

int p_set_body_add( World* w, int setId, int bodyId )
{
	SolverSet* s = set_get( w, setId );
	Body* b = w->bodies + bodyId;
	b->setIndex = setId;
	b->localIndex = s->bodies.count;
	ia_push( &s->bodies, bodyId );
	return b->localIndex;
}

static void set_body_remove( World* w, int setId, int bodyId )
{
	SolverSet* s = set_get( w, setId );
	Body* b = w->bodies + bodyId;
	int idx = b->localIndex;
	int moved = ia_remove_swap( &s->bodies, idx );
	if ( moved != P_NULL )
		w->bodies[s->bodies.data[idx]].localIndex = idx;
	b->localIndex = P_NULL;
}

int p_body_awake( const World* w, int bodyId )
{
	return w->bodies[bodyId].setIndex == SET_AWAKE;
}

// ---------------------------------------------------------------------------
// islands (island.c)
// ---------------------------------------------------------------------------
static Island* island_get( World* w, int id )
{
	return w->islands + id;
}

// island.c:18-56
static int island_create( World* w, int setId )
{
	int id = pool_alloc( &w->islandPool );
	if ( id >= w->islandCap )
	{
		int cap = w->islandCap < 16 ? 16 : 2 * w->islandCap;
		while ( cap <= id )
			cap *= 2;
		w->islands = (Island*)realloc( w->islands, sizeof( Island ) * (size_t)cap );
		w->islandCap = cap;
	}
	SolverSet* s = set_get( w, setId );
	Island* isl = w->islands + id;
	isl->setIndex = setId;
	isl->localIndex = s->islands.count;
	isl->islandId = id;
	isl->headBody = isl->tailBody = P_NULL;
	isl->bodyCount = 0;
	isl->headContact = isl->tailContact = P_NULL;
	isl->contactCount = 0;
	isl->headJoint = isl->tailJoint = P_NULL;
	isl->jointCount = 0;
	isl->parentIsland = P_NULL;
	isl->constraintRemoveCount = 0;
	ia_push( &s->islands, id );
	return id;
}

// island.c:58-84
static void island_destroy( World* w, int id )
{
	if ( w->splitIslandId == id )
		w->splitIslandId = P_NULL;
	Island* isl = island_get( w, id );
	SolverSet* s = set_get( w, isl->setIndex );
	int moved = ia_remove_swap( &s->islands, isl->localIndex );
	if ( moved != P_NULL )
		w->islands[s->islands.data[isl->localIndex]].localIndex = isl->localIndex;
	isl->islandId = P_NULL;
	isl->setIndex = P_NULL;
	isl->localIndex = P_NULL;
	pool_free( &w->islandPool, id );
}

// body.c:84-96
void p_create_island_for_body( World* w, int setId, int bodyId )
{
	int id = island_create( w, setId );
	Island* isl = island_get( w, id );
	Body* b = w->bodies + bodyId;
	b->islandId = id;
	b->islandPrev = b->islandNext = P_NULL;
	isl->headBody = bodyId;
	isl->tailBody = bodyId;
	isl->bodyCount = 1;
}

// union-find root with path compression (island.c:150-196); compression
// never changes a root
static int island_root( World* w, int id )
{
	while ( w->islands[id].parentIsland != P_NULL )
	{
		Island* isl = w->islands + id;
		int parentId = isl->parentIsland;
		Island* parent = w->islands + parentId;
		if ( parent->parentIsland != P_NULL )
			isl->parentIsland = parent->parentIsland;
		id = parentId;
	}
	return id;
}

// island.c:86-110: new contact at the head of the island's list
static void island_add_contact( World* w, int islandId, int cid )
{
	Island* isl = island_get( w, islandId );
	Contact* c = w->contacts + cid;
	if ( isl->headContact != P_NULL )
	{
		c->islandNext = isl->headContact;
		w->contacts[isl->headContact].islandPrev = cid;
	}
	isl->headContact = cid;
	if ( isl->tailContact == P_NULL )
		isl->tailContact = isl->headContact;
	isl->contactCount += 1;
	c->islandId = islandId;
}

// island.c:116-218
void p_link_contact( World* w, int cid )
{
	Contact* c = w->contacts + cid;
	Body* a = w->bodies + c->bodyA;
	Body* b = w->bodies + c->bodyB;
	if ( a->setIndex == SET_AWAKE && b->setIndex >= SET_FIRST_SLEEPING )
		p_wake_solver_set( w, b->setIndex );
	if ( b->setIndex == SET_AWAKE && a->setIndex >= SET_FIRST_SLEEPING )
		p_wake_solver_set( w, a->setIndex );
	int idA = a->islandId, idB = b->islandId;
	if ( idA == idB )
	{
		island_add_contact( w, idA, cid );
		return;
	}
	int rootA = idA != P_NULL ? island_root( w, idA ) : P_NULL;
	int rootB = idB != P_NULL ? island_root( w, idB ) : P_NULL;
	if ( rootA != rootB && rootA != P_NULL && rootB != P_NULL )
		island_get( w, rootB )->parentIsland = rootA;
	if ( rootA != P_NULL )
		island_add_contact( w, rootA, cid );
	else
		island_add_contact( w, rootB, cid );
}

// island.c:221-261
void p_unlink_contact( World* w, int cid )
{
	Contact* c = w->contacts + cid;
	int id = c->islandId;
	Island* isl = island_get( w, id );
	if ( c->islandPrev != P_NULL )
		w->contacts[c->islandPrev].islandNext = c->islandNext;
	if ( c->islandNext != P_NULL )
		w->contacts[c->islandNext].islandPrev = c->islandPrev;
	if ( isl->headContact == cid )
		isl->headContact = c->islandNext;
	if ( isl->tailContact == cid )
		isl->tailContact = c->islandPrev;
	isl->contactCount -= 1;
	isl->constraintRemoveCount += 1;
	c->islandId = c->islandPrev = c->islandNext = P_NULL;
}

// island.c:264-289
static void island_add_joint( World* w, int islandId, int jid )
{
	Island* isl = island_get( w, islandId );
	Joint* j = w->joints + jid;
	if ( isl->headJoint != P_NULL )
	{
		j->islandNext = isl->headJoint;
		w->joints[isl->headJoint].islandPrev = jid;
	}
	isl->headJoint = jid;
	if ( isl->tailJoint == P_NULL )
		isl->tailJoint = isl->headJoint;
	isl->jointCount += 1;
	j->islandId = islandId;
}

// island.c:291-382
void p_link_joint( World* w, int jid, int mergeIslands )
{
	Joint* j = w->joints + jid;
	Body* a = w->bodies + j->bodyA;
	Body* b = w->bodies + j->bodyB;
	if ( a->setIndex == SET_AWAKE && b->setIndex >= SET_FIRST_SLEEPING )
		p_wake_solver_set( w, b->setIndex );
	else if ( b->setIndex == SET_AWAKE && a->setIndex >= SET_FIRST_SLEEPING )
		p_wake_solver_set( w, a->setIndex );
	int idA = a->islandId, idB = b->islandId;
	if ( idA == idB )
	{
		island_add_joint( w, idA, jid );
		return;
	}
	int rootA = idA != P_NULL ? island_root( w, idA ) : P_NULL;
	int rootB = idB != P_NULL ? island_root( w, idB ) : P_NULL;
	if ( rootA != rootB && rootA != P_NULL && rootB != P_NULL )
		island_get( w, rootB )->parentIsland = rootA;
	if ( rootA != P_NULL )
		island_add_joint( w, rootA, jid );
	else
		island_add_joint( w, rootB, jid );
	if ( mergeIslands )
		p_merge_awake_islands( w );
}

// island.c:429-528: append the island's lists to its root's
static void island_merge( World* w, Island* isl )
{
	int rootId = isl->parentIsland;
	Island* root = island_get( w, rootId );
	for ( int b = isl->headBody; b != P_NULL; b = w->bodies[b].islandNext )
		w->bodies[b].islandId = rootId;
	for ( int c = isl->headContact; c != P_NULL; c = w->contacts[c].islandNext )
		w->contacts[c].islandId = rootId;
	for ( int j = isl->headJoint; j != P_NULL; j = w->joints[j].islandNext )
		w->joints[j].islandId = rootId;

	w->bodies[root->tailBody].islandNext = isl->headBody;
	w->bodies[isl->headBody].islandPrev = root->tailBody;
	root->tailBody = isl->tailBody;
	root->bodyCount += isl->bodyCount;

	if ( root->headContact == P_NULL )
	{
		root->headContact = isl->headContact;
		root->tailContact = isl->tailContact;
		root->contactCount = isl->contactCount;
	}
	else if ( isl->headContact != P_NULL )
	{
		w->contacts[root->tailContact].islandNext = isl->headContact;
		w->contacts[isl->headContact].islandPrev = root->tailContact;
		root->tailContact = isl->tailContact;
		root->contactCount += isl->contactCount;
	}

	if ( root->headJoint == P_NULL )
	{
		root->headJoint = isl->headJoint;
		root->tailJoint = isl->tailJoint;
		root->jointCount = isl->jointCount;
	}
	else if ( isl->headJoint != P_NULL )
	{
		w->joints[root->tailJoint].islandNext = isl->headJoint;
		w->joints[isl->headJoint].islandPrev = root->tailJoint;
		root->tailJoint = isl->tailJoint;
		root->jointCount += isl->jointCount;
	}
	root->constraintRemoveCount += isl->constraintRemoveCount;
}

// island.c:539-600
void p_merge_awake_islands( World* w )
{
	SolverSet* awake = set_get( w, SET_AWAKE );
	int n = awake->islands.count;
	for ( int i = 0; i < n; ++i )
	{
		int id = awake->islands.data[i];
		Island* isl = island_get( w, id );
		int root = island_root( w, id );
		if ( root != id )
			isl->parentIsland = root;
	}
	for ( int i = n - 1; i >= 0; --i )
	{
		int id = awake->islands.data[i];
		Island* isl = island_get( w, id );
		if ( isl->parentIsland == P_NULL )
			continue;
		island_merge( w, isl );
		island_destroy( w, id );
	}
}

// island.c:602-832: depth-first search from every body of the base island
void p_split_island( World* w, int baseId )
{
	Island* base = island_get( w, baseId );
	int setId = base->setIndex;
	if ( setId != SET_AWAKE || base->constraintRemoveCount == 0 )
		return;
	int bodyCount = base->bodyCount;
	int* stack = (int*)malloc( sizeof( int ) * (size_t)( bodyCount > 0 ? bodyCount : 1 ) );
	int* bodyIds = (int*)malloc( sizeof( int ) * (size_t)( bodyCount > 0 ? bodyCount : 1 ) );
	int index = 0;
	for ( int b = base->headBody; b != P_NULL; b = w->bodies[b].islandNext )
	{
		bodyIds[index++] = b;
		w->bodies[b].isMarked = 0;
	}
	for ( int c = base->headContact; c != P_NULL; c = w->contacts[c].islandNext )
		w->contacts[c].isMarked = 0;
	for ( int j = base->headJoint; j != P_NULL; j = w->joints[j].islandNext )
		w->joints[j].isMarked = 0;
	island_destroy( w, baseId );

	for ( int i = 0; i < bodyCount; ++i )
	{
		int seed = bodyIds[i];
		if ( w->bodies[seed].isMarked )
			continue;
		int sp = 0;
		stack[sp++] = seed;
		w->bodies[seed].isMarked = 1;
		int id = island_create( w, setId );
		Island* isl = island_get( w, id );
		while ( sp > 0 )
		{
			int bodyId = stack[--sp];
			Body* body = w->bodies + bodyId;
			body->islandId = id;
			if ( isl->tailBody != P_NULL )
				w->bodies[isl->tailBody].islandNext = bodyId;
			body->islandPrev = isl->tailBody;
			body->islandNext = P_NULL;
			isl->tailBody = bodyId;
			if ( isl->headBody == P_NULL )
				isl->headBody = bodyId;
			isl->bodyCount += 1;

			for ( int key = body->headContactKey; key != P_NULL; )
			{
				int cid = key >> 1, edge = key & 1;
				Contact* c = w->contacts + cid;
				key = c->edgeNext[edge];
				if ( c->isMarked )
					continue;
				if ( c->touchingFlag == 0 )
					continue;
				c->isMarked = 1;
				int other = edge == 0 ? c->bodyB : c->bodyA;
				Body* ob = w->bodies + other;
				if ( ob->isMarked == 0 && ob->setIndex != SET_STATIC )
				{
					stack[sp++] = other;
					ob->isMarked = 1;
				}
				c->islandId = id;
				if ( isl->tailContact != P_NULL )
					w->contacts[isl->tailContact].islandNext = cid;
				c->islandPrev = isl->tailContact;
				c->islandNext = P_NULL;
				isl->tailContact = cid;
				if ( isl->headContact == P_NULL )
					isl->headContact = cid;
				isl->contactCount += 1;
			}

			for ( int key = body->headJoint; key != P_NULL; )
			{
				int jid = key >> 1, edge = key & 1;
				Joint* j = w->joints + jid;
				key = edge == 0 ? j->nextA : j->nextB;
				if ( j->isMarked )
					continue;
				j->isMarked = 1;
				int other = edge == 0 ? j->bodyB : j->bodyA;
				Body* ob = w->bodies + other;
				if ( ob->setIndex == SET_DISABLED )
					continue;
				if ( ob->isMarked == 0 && ob->setIndex == SET_AWAKE )
				{
					stack[sp++] = other;
					ob->isMarked = 1;
				}
				j->islandId = id;
				if ( isl->tailJoint != P_NULL )
					w->joints[isl->tailJoint].islandNext = jid;
				j->islandPrev = isl->tailJoint;
				j->islandNext = P_NULL;
				isl->tailJoint = jid;
				if ( isl->headJoint == P_NULL )
					isl->headJoint = jid;
				isl->jointCount += 1;
			}
		}
	}
	free( bodyIds );
	free( stack );
}

// ---------------------------------------------------------------------------
// body contact edge lists (contact.c:240-283 create, :355-410 destroy)
// ---------------------------------------------------------------------------
void p_contact_edges_link( World* w, int cid )
{
	Contact* c = w->contacts + cid;
	for ( int e = 0; e < 2; ++e )
	{
		Body* b = w->bodies + ( e == 0 ? c->bodyA : c->bodyB );
		int key = ( cid << 1 ) | e;
		c->edgePrev[e] = P_NULL;
		c->edgeNext[e] = b->headContactKey;
		if ( b->headContactKey != P_NULL )
		{
			int h = b->headContactKey;
			w->contacts[h >> 1].edgePrev[h & 1] = key;
		}
		b->headContactKey = key;
		b->contactCount += 1;
	}
}

void p_contact_edges_unlink( World* w, int cid )
{
	Contact* c = w->contacts + cid;
	for ( int e = 0; e < 2; ++e )
	{
		Body* b = w->bodies + ( e == 0 ? c->bodyA : c->bodyB );
		if ( c->edgePrev[e] != P_NULL )
		{
			int p = c->edgePrev[e];
			w->contacts[p >> 1].edgeNext[p & 1] = c->edgeNext[e];
		}
		if ( c->edgeNext[e] != P_NULL )
		{
			int n = c->edgeNext[e];
			w->contacts[n >> 1].edgePrev[n & 1] = c->edgePrev[e];
		}
		int key = ( cid << 1 ) | e;
		if ( b->headContactKey == key )
			b->headContactKey = c->edgeNext[e];
		b->contactCount -= 1;
		c->edgePrev[e] = c->edgeNext[e] = P_NULL;
	}
}

// ---------------------------------------------------------------------------
// sleeping and waking (solver_set.c)
// ---------------------------------------------------------------------------
// solver_set.c:36-147
void p_wake_solver_set( World* w, int setId )
{
	SolverSet* set = set_get( w, setId );
	int bodyCount = set->bodies.count;
	for ( int i = 0; i < bodyCount; ++i )
	{
		int bodyId = w->sets[setId].bodies.data[i];
		Body* b = w->bodies + bodyId;
		p_set_body_add( w, SET_AWAKE, bodyId );
		b->sleepTime = 0.0f;
		// b2_identityBodyState
		b->v = V( 0.0f, 0.0f );
		b->w = 0.0f;
		b->dp = V( 0.0f, 0.0f );
		b->dq.c = 1.0f;
		b->dq.s = 0.0f;
		for ( int key = b->headContactKey; key != P_NULL; )
		{
			Contact* c = w->contacts + ( key >> 1 );
			key = c->edgeNext[key & 1];
			if ( c->setIndex != SET_DISABLED )
				continue;
			c->setIndex = SET_AWAKE;
		}
	}
	set = set_get( w, setId );
	for ( int i = 0; i < set->contacts.count; ++i )
	{
		int cid = set->contacts.data[i];
		p_add_contact_to_graph( w, cid );
		w->contacts[cid].setIndex = SET_AWAKE;
	}
	for ( int i = 0; i < set->joints.count; ++i )
	{
		int jid = set->joints.data[i];
		p_add_joint_to_graph( w, jid );
		w->joints[jid].setIndex = SET_AWAKE;
	}
	SolverSet* awake = set_get( w, SET_AWAKE );
	for ( int i = 0; i < set->islands.count; ++i )
	{
		int id = set->islands.data[i];
		Island* isl = island_get( w, id );
		isl->setIndex = SET_AWAKE;
		isl->localIndex = awake->islands.count;
		ia_push( &awake->islands, id );
	}
	set_destroy( w, setId );
}

// solver_set.c:156-414
void p_try_sleep_island( World* w, int islandId )
{
	Island* isl = island_get( w, islandId );
	if ( isl->constraintRemoveCount > 0 )
		return;
	int sleepId = set_create( w );
	isl = island_get( w, islandId );

	for ( int bodyId = isl->headBody; bodyId != P_NULL; )
	{
		Body* b = w->bodies + bodyId;
		if ( b->moveEventIndex != P_NULL )
		{
			w->moveEventAsleep[b->moveEventIndex] = 1;
			b->moveEventIndex = P_NULL;
		}
		set_body_remove( w, SET_AWAKE, bodyId );
		p_set_body_add( w, sleepId, bodyId );
		// the body state leaves with the awake set (solver_set.c:225): a
		// sleeping body reads zero velocity
		b->v = V( 0.0f, 0.0f );
		b->w = 0.0f;
		b->dp = V( 0.0f, 0.0f );
		b->dq.c = 1.0f;
		b->dq.s = 0.0f;
		for ( int key = b->headContactKey; key != P_NULL; )
		{
			int cid = key >> 1, edge = key & 1;
			Contact* c = w->contacts + cid;
			key = c->edgeNext[edge];
			if ( c->setIndex == SET_DISABLED )
				continue;
			if ( c->color != P_NULL )
				continue;
			int other = edge == 0 ? c->bodyB : c->bodyA;
			if ( w->bodies[other].setIndex == SET_AWAKE )
				continue;
			c->setIndex = SET_DISABLED;
		}
		bodyId = b->islandNext;
	}

	for ( int cid = isl->headContact; cid != P_NULL; )
	{
		Contact* c = w->contacts + cid;
		p_remove_contact_from_graph( w, cid );
		ia_push( &set_get( w, sleepId )->contacts, cid );
		c->setIndex = sleepId;
		cid = c->islandNext;
	}

	for ( int jid = isl->headJoint; jid != P_NULL; )
	{
		Joint* j = w->joints + jid;
		p_remove_joint_from_graph( w, jid );
		ia_push( &set_get( w, sleepId )->joints, jid );
		j->setIndex = sleepId;
		jid = j->islandNext;
	}

	SolverSet* awake = set_get( w, SET_AWAKE );
	int moved = ia_remove_swap( &awake->islands, isl->localIndex );
	if ( moved != P_NULL )
		w->islands[awake->islands.data[isl->localIndex]].localIndex = isl->localIndex;
	ia_push( &set_get( w, sleepId )->islands, islandId );
	isl->setIndex = sleepId;
	isl->localIndex = 0;
}

// solver.c:2003-2048 with one task context: the split candidate is chosen
// by the caller; islands whose bit is clear try to sleep, last first.
void p_sleep_islands( World* w, const unsigned char* awakeIslandBits, int splitCandidate )
{
	w->splitIslandId = splitCandidate;
	SolverSet* awake = set_get( w, SET_AWAKE );
	for ( int i = awake->islands.count - 1; i >= 0; --i )
	{
		if ( awakeIslandBits[i] )
			continue;
		int id = set_get( w, SET_AWAKE )->islands.data[i];
		p_try_sleep_island( w, id );
	}
}

int p_new_sleeping_set( World* w )
{
	return set_create( w );
}

void p_set_joint_add( World* w, int setId, int jid )
{
	ia_push( &set_get( w, setId )->joints, jid );
	w->joints[jid].setIndex = setId;
}

// solver_set.c:419-517: the set with fewer bodies moves into the other
void p_merge_solver_sets( World* w, int setId1, int setId2 )
{
	if ( w->sets[setId1].bodies.count < w->sets[setId2].bodies.count )
	{
		int t = setId1;
		setId1 = setId2;
		setId2 = t;
	}
	SolverSet* s2 = set_get( w, setId2 );
	for ( int i = 0; i < s2->bodies.count; ++i )
		p_set_body_add( w, setId1, s2->bodies.data[i] );
	for ( int i = 0; i < s2->contacts.count; ++i )
	{
		int cid = s2->contacts.data[i];
		w->contacts[cid].setIndex = setId1;
		ia_push( &set_get( w, setId1 )->contacts, cid );
	}
	for ( int i = 0; i < s2->joints.count; ++i )
	{
		int jid = s2->joints.data[i];
		w->joints[jid].setIndex = setId1;
		ia_push( &set_get( w, setId1 )->joints, jid );
	}
	for ( int i = 0; i < s2->islands.count; ++i )
	{
		int id = s2->islands.data[i];
		SolverSet* s1 = set_get( w, setId1 );
		w->islands[id].setIndex = setId1;
		w->islands[id].localIndex = s1->islands.count;
		ia_push( &s1->islands, id );
	}
	set_destroy( w, setId2 );
}

// ---------------------------------------------------------------------------
// removal (the destroy path, pdestroy.c)
// ---------------------------------------------------------------------------
// island.c:384-424 b2UnlinkJoint
void p_unlink_joint( World* w, int jid )
{
	Joint* j = w->joints + jid;
	Island* isl = island_get( w, j->islandId );
	if ( j->islandPrev != P_NULL )
		w->joints[j->islandPrev].islandNext = j->islandNext;
	if ( j->islandNext != P_NULL )
		w->joints[j->islandNext].islandPrev = j->islandPrev;
	if ( isl->headJoint == jid )
		isl->headJoint = j->islandNext;
	if ( isl->tailJoint == jid )
		isl->tailJoint = j->islandPrev;
	isl->jointCount -= 1;
	isl->constraintRemoveCount += 1;
	j->islandId = j->islandPrev = j->islandNext = P_NULL;
}

// body.c:99-157 b2RemoveBodyFromIsland: an island left without bodies is
// destroyed
void p_remove_body_from_island( World* w, int bodyId )
{
	Body* b = w->bodies + bodyId;
	if ( b->islandId == P_NULL )
		return;
	int id = b->islandId;
	Island* isl = island_get( w, id );
	if ( b->islandPrev != P_NULL )
		w->bodies[b->islandPrev].islandNext = b->islandNext;
	if ( b->islandNext != P_NULL )
		w->bodies[b->islandNext].islandPrev = b->islandPrev;
	isl->bodyCount -= 1;
	if ( isl->headBody == bodyId )
	{
		isl->headBody = b->islandNext;
		if ( isl->headBody == P_NULL )
			island_destroy( w, id );
	}
	else if ( isl->tailBody == bodyId )
		isl->tailBody = b->islandPrev;
	b->islandId = b->islandPrev = b->islandNext = P_NULL;
}

// body.c:412-432: swap-remove from the owning set; a sleeping set left
// without bodies is destroyed (solver_set.c:18-29)
void p_set_remove_body( World* w, int bodyId )
{
	Body* b = w->bodies + bodyId;
	int setId = b->setIndex;
	if ( setId == P_NULL )
		return;
	set_body_remove( w, setId, bodyId );
	if ( setId >= SET_FIRST_SLEEPING && set_get( w, setId )->bodies.count == 0 )
		set_destroy( w, setId );
	b->setIndex = P_NULL;
}

// solver_set.c:521-556 b2TransferBody: the body joins the target set's
// array and leaves the source set's by swap-remove; a body entering the awake
// set gets the identity state and one leaving it loses its state (velocity)
void p_transfer_body( World* w, int targetSet, int bodyId )
{
	Body* b = w->bodies + bodyId;
	int src = b->setIndex;
	set_body_remove( w, src, bodyId );
	p_set_body_add( w, targetSet, bodyId );
	if ( src == SET_AWAKE || targetSet == SET_AWAKE )
	{
		b->v = V( 0.0f, 0.0f );
		b->w = 0.0f;
		b->dp = V( 0.0f, 0.0f );
		b->dq.c = 1.0f;
		b->dq.s = 0.0f;
	}
}

static void remove_swap_value( IntArr* a, int v )
{
	for ( int i = 0; i < a->count; ++i )
		if ( a->data[i] == v )
		{
			ia_remove_swap( a, i );
			return;
		}
}

// contact.c:428-440 / joint.c:774-787: a constraint outside the constraint
// graph leaves its set's array by swap-remove
void p_set_remove_contact( World* w, int cid )
{
	int setId = w->contacts[cid].setIndex;
	if ( setId != P_NULL && setId != SET_AWAKE && setId < w->setCap )
		remove_swap_value( &set_get( w, setId )->contacts, cid );
}

void p_set_remove_joint( World* w, int jid )
{
	int setId = w->joints[jid].setIndex;
	if ( setId != P_NULL && setId != SET_AWAKE && setId < w->setCap )
		remove_swap_value( &set_get( w, setId )->joints, jid );
}

// body.c:331-340 b2WakeBody
int p_wake_body( World* w, int bodyId )
{
	int setId = w->bodies[bodyId].setIndex;
	if ( setId >= SET_FIRST_SLEEPING )
	{
		p_wake_solver_set( w, setId );
		return 1;
	}
	return 0;
}

// solver_set.c:558-613 b2TransferJoint: out of the constraint graph (awake)
// or the source set's array (swap-remove), into the graph (awake) or the
// target set's array (appended)
void p_transfer_joint( World* w, int targetSet, int jid )
{
	Joint* j = w->joints + jid;
	if ( j->setIndex == SET_AWAKE )
		p_remove_joint_from_graph( w, jid );
	else
		p_set_remove_joint( w, jid );
	if ( targetSet == SET_AWAKE )
	{
		j->setIndex = SET_AWAKE;
		p_add_joint_to_graph( w, jid );
	}
	else
		p_set_joint_add( w, targetSet, jid );
}
