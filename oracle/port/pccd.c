// Continuous collision of fast non-bullet bodies against static shapes.
// TEST INFRASTRUCTURE (oracle). Restates solver.c:196-388
// (b2ContinuousQueryCallback) and :390-541 (b2SolveContinuous) of
// packages/forge2d/third_party/box2d/src. Candidate static shapes are
// visited in the static tree's depth-first order (p_static_order), as the
// reference's query meets them: the running fraction narrows with each hit,
// so the order shows in the last bits of the result.
#include "port.h"

static int should_collide_filters( const Shape* a, const Shape* b )
{
	if ( a->groupIndex == b->groupIndex && a->groupIndex != 0 )
		return a->groupIndex > 0;
	return ( a->maskBits & b->categoryBits ) != 0 && ( a->categoryBits & b->maskBits ) != 0;
}

static Sweep make_sweep( const Body* b )
{
	Sweep s;
	s.c1 = b->center0;
	s.c2 = b->center;
	s.q1 = b->rotation0;
	s.q2 = b->xf.q;
	s.localCenter = b->localCenter;
	return s;
}

// joint exclusion as body.c:1861-1897 (pairs with a static body are never
// dynamic-dynamic, so only the joint list matters)
static int bodies_collide( World* w, int ia, int ib )
{
	Body* a = w->bodies + ia;
	Body* b = w->bodies + ib;
	if ( a->type != BODY_DYNAMIC && b->type != BODY_DYNAMIC )
		return 0;
	int key, other;
	if ( a->jointCount < b->jointCount )
	{
		key = a->headJoint;
		other = ib;
	}
	else
	{
		key = b->headJoint;
		other = ia;
	}
	while ( key != P_NULL )
	{
		int jid = key >> 1;
		int edge = key & 1;
		Joint* j = w->joints + jid;
		int otherBody = edge == 0 ? j->bodyB : j->bodyA;
		if ( j->collideConnected == 0 && otherBody == other )
			return 0;
		key = edge == 0 ? j->nextA : j->nextB;
	}
	return 1;
}

void p_solve_continuous( World* w, int bodyId )
{
	Body* fast = w->bodies + bodyId;
	Sweep sweep = make_sweep( fast );
	xform xf1;
	xf1.q = sweep.q1;
	xf1.p = sub( sweep.c1, rotate( sweep.q1, sweep.localCenter ) );
	xform xf2;
	xf2.q = sweep.q2;
	xf2.p = sub( sweep.c2, rotate( sweep.q2, sweep.localCenter ) );
	float fraction = 1.0f;
	for ( int fs = fast->headShape; fs != P_NULL; fs = w->shapes[fs].nextShape )
	{
		Shape* fastShape = w->shapes + fs;
		box2 box1 = fastShape->aabb;
		box2 box2v = p_shape_aabb( &fastShape->g, xf2 );
		box2 box = boxUnion( box1, box2v );
		fastShape->aabb = box2v;
		if ( fastShape->isSensor )
			continue;
		v2 centroid1 = xfPoint( xf1, fastShape->localCentroid );
		v2 centroid2 = xfPoint( xf2, fastShape->localCentroid );
		for ( int k = 0; k < w->staticOrderCount; ++k )
		{
			int si = w->staticOrder[k];
			Shape* shape = w->shapes + si;
			if ( shape->used == 0 || shape->proxyKey == P_NULL || ( shape->proxyKey & 3 ) != BODY_STATIC )
				continue;
			if ( boxOverlaps( shape->fatAABB, box ) == 0 )
				continue;
			if ( si == fs || shape->bodyId == fastShape->bodyId || shape->isSensor || shape->sub != fastShape->sub )
				continue;
			if ( should_collide_filters( fastShape, shape ) == 0 )
				continue;
			Body* body = w->bodies + shape->bodyId;
			if ( body->isBullet )
				continue;
			if ( bodies_collide( w, bodyId, shape->bodyId ) == 0 )
				continue;
			// solver.c:270-280 the custom filter (static shape first)
			if ( w->customFilter && w->customFilter( si, fs, w->customFilterContext ) == 0 )
				continue;
			// solver.c:283-304: no pausing on chain segment junctions (the fast
			// shape starts behind, or crosses by less than a quarter of the
			// body's minimum extent)
			if ( shape->g.type == SHAPE_CHAIN_SEGMENT )
			{
				xform transform = body->xf;
				v2 p1 = xfPoint( transform, shape->g.c1 );
				v2 p2 = xfPoint( transform, shape->g.c2 );
				float len;
				v2 e = lengthAndNormalize( &len, sub( p2, p1 ) );
				if ( len > P_LINEAR_SLOP )
				{
					float offset1 = cross( sub( centroid1, p1 ), e );
					float offset2 = cross( sub( centroid2, p1 ), e );
					const float allowedFraction = 0.25f;
					if ( offset1 < 0.0f || offset1 - offset2 < allowedFraction * fast->minExtent )
						continue;
				}
			}
			ShapeProxy pa = p_shape_proxy( &shape->g );
			ShapeProxy pb = p_shape_proxy( &fastShape->g );
			Sweep sa = make_sweep( body );
			int state;
			float hitFraction = fraction;
			int didHit = 0;
			float f = p_time_of_impact( &pa, &pb, sa, sweep, fraction, &state );
			if ( 0.0f < f && f < fraction )
			{
				hitFraction = f;
				didHit = 1;
			}
			else if ( 0.0f == f )
			{
				v2 centroid = p_shape_centroid( &fastShape->g );
				float mn, mx;
				p_shape_extent( fastShape, centroid, &mn, &mx );
				float radius = 0.25f * mn;
				ShapeProxy pc = p_make_proxy( &centroid, 1, radius );
				f = p_time_of_impact( &pa, &pc, sa, sweep, fraction, &state );
				if ( 0.0f < f && f < fraction )
				{
					hitFraction = f;
					didHit = 1;
				}
			}
			if ( didHit )
				fraction = hitFraction;
		}
	}
	if ( fraction < 1.0f )
	{
		rot q = nlerpRot( sweep.q1, sweep.q2, fraction );
		v2 c = lerp( sweep.c1, sweep.c2, fraction );
		v2 origin = sub( c, rotate( q, sweep.localCenter ) );
		xform transform = { origin, q };
		fast->xf = transform;
		fast->center = c;
		fast->rotation0 = q;
		fast->center0 = c;
		// the move event of this body was already written with the
		// unadvanced transform; patch it (solver.c:472-474)
		if ( w->moveEventBodies[fast->moveEventIndex] == bodyId )
		{
			float* x = w->moveEventXf + 4 * fast->moveEventIndex;
			x[0] = transform.p.x;
			x[1] = transform.p.y;
			x[2] = transform.q.c;
			x[3] = transform.q.s;
		}
		for ( int s = fast->headShape; s != P_NULL; s = w->shapes[s].nextShape )
		{
			Shape* sh = w->shapes + s;
			box2 aabb = p_shape_aabb( &sh->g, transform );
			aabb.lo.x -= P_SPECULATIVE;
			aabb.lo.y -= P_SPECULATIVE;
			aabb.hi.x += P_SPECULATIVE;
			aabb.hi.y += P_SPECULATIVE;
			sh->aabb = aabb;
			if ( boxContains( sh->fatAABB, aabb ) == 0 )
			{
				box2 fat;
				fat.lo.x = aabb.lo.x - P_AABB_MARGIN;
				fat.lo.y = aabb.lo.y - P_AABB_MARGIN;
				fat.hi.x = aabb.hi.x + P_AABB_MARGIN;
				fat.hi.y = aabb.hi.y + P_AABB_MARGIN;
				sh->fatAABB = fat;
				sh->enlarged = 1;
				fast->enlargeAABB = 1;
			}
		}
	}
	else
	{
		fast->rotation0 = fast->xf.q;
		fast->center0 = fast->center;
		for ( int s = fast->headShape; s != P_NULL; s = w->shapes[s].nextShape )
		{
			Shape* sh = w->shapes + s;
			if ( boxContains( sh->fatAABB, sh->aabb ) == 0 )
			{
				box2 fat;
				fat.lo.x = sh->aabb.lo.x - P_AABB_MARGIN;
				fat.lo.y = sh->aabb.lo.y - P_AABB_MARGIN;
				fat.hi.x = sh->aabb.hi.x + P_AABB_MARGIN;
				fat.hi.y = sh->aabb.hi.y + P_AABB_MARGIN;
				sh->fatAABB = fat;
				sh->enlarged = 1;
				fast->enlargeAABB = 1;
			}
		}
	}
}
