// Sensor overlaps and events of the restatement. TEST INFRASTRUCTURE
// (oracle). Reference: packages/forge2d/third_party/box2d/src/sensor.c:48-334
// (b2SensorQueryCallback, b2SensorTask, b2OverlapSensors), run at the end of
// the step (world.c:788-793).
//
// A sensor whose body is enabled and whose enableSensorEvents is set
// overlaps every other shape that has a proxy whose fat AABB meets the
// sensor's AABB (the trees' query, category & the sensor's mask), has
// enableSensorEvents, sits on another body, passes the filter and whose
// GJK distance with radii is below 10 FLT_EPSILON. The overlaps are sorted
// by shape id; a sensor whose sorted set changed reports, in sensor order,
// the ends and begins of a merge of the old and the new set.
#include "port.h"

#include <stdlib.h>

static int cmp_int( const void* a, const void* b )
{
	int x = *(const int*)a, y = *(const int*)b;
	return x < y ? -1 : ( x > y ? 1 : 0 );
}

// shape.c:1625-1648 b2ShouldShapesCollide
static int filters_collide( const Shape* a, const Shape* b )
{
	if ( a->groupIndex == b->groupIndex && a->groupIndex != 0 )
		return a->groupIndex > 0;
	return ( a->maskBits & b->categoryBits ) != 0 && ( a->categoryBits & b->maskBits ) != 0;
}

// distance.c:421-606 with useRadii = true
static float distance_with_radii( const Shape* a, xform xfA, const Shape* b, xform xfB )
{
	ShapeProxy pa = p_shape_proxy( &a->g );
	ShapeProxy pb = p_shape_proxy( &b->g );
	SimplexCache cache = { 0 };
	float d = p_shape_distance( &pa, &pb, xfA, xfB, &cache, NULL, NULL, NULL );
	if ( d > 0.1f * P_LINEAR_SLOP )
	{
		d = d - pa.radius - pb.radius;
		d = d > 0.0f ? d : 0.0f;
	}
	return d;
}

void p_overlap_sensors( World* w )
{
	for ( int k = 0; k < w->sensorCount; ++k )
	{
		PSensor* sn = w->sensors + k;
		IntArr t = sn->overlaps1;
		sn->overlaps1 = sn->overlaps2;
		sn->overlaps2 = t;
		sn->overlaps2.count = 0;
		const Shape* ss = w->shapes + sn->shapeId;
		const Body* body = w->bodies + ss->bodyId;
		if ( body->enabled && ss->enableSensorEvents )
		{
			xform xf = body->xf;
			for ( int id = 0; id < w->shapeCount; ++id )
			{
				const Shape* o = w->shapes + id;
				if ( o->used == 0 || o->proxyKey == P_NULL || id == sn->shapeId )
					continue;
				if ( ( o->categoryBits & ss->maskBits ) == 0 || boxOverlaps( o->fatAABB, ss->aabb ) == 0 )
					continue;
				if ( o->enableSensorEvents == 0 || o->bodyId == ss->bodyId || filters_collide( ss, o ) == 0 )
					continue;
				if ( distance_with_radii( ss, xf, o, w->bodies[o->bodyId].xf ) < 10.0f * FLT_EPSILON )
					ia_push( &sn->overlaps2, id );
			}
			qsort( sn->overlaps2.data, (size_t)sn->overlaps2.count, sizeof( int ), cmp_int );
		}
		// merge (shapes are never destroyed here, so generations agree)
		const int* r1 = sn->overlaps1.data;
		const int* r2 = sn->overlaps2.data;
		int n1 = sn->overlaps1.count, n2 = sn->overlaps2.count;
		int i1 = 0, i2 = 0;
		while ( i1 < n1 || i2 < n2 )
		{
			if ( i2 == n2 || ( i1 < n1 && r1[i1] < r2[i2] ) )
			{
				ia_push( &w->sensorEnd, sn->shapeId );
				ia_push( &w->sensorEnd, r1[i1++] );
			}
			else if ( i1 == n1 || r2[i2] < r1[i1] )
			{
				ia_push( &w->sensorBegin, sn->shapeId );
				ia_push( &w->sensorBegin, r2[i2++] );
			}
			else
			{
				i1 += 1;
				i2 += 1;
			}
		}
	}
}
