// World queries of the restatement: closest ray hit and AABB overlap.
// TEST INFRASTRUCTURE (oracle).
//
// Reference (packages/forge2d/third_party/box2d/src/):
//   world.c:2050-2098  b2World_OverlapAABB: every proxy whose tree box (the
//                      fat AABB) overlaps the query box and whose filter
//                      passes b2ShouldQueryCollide (shape.h:132-135)
//   world.c:2185-2310  b2World_CastRayClosest: ray against the shapes in the
//                      three trees, hits at fraction 0 (initial overlap)
//                      ignored, the closest hit kept
//   shape.c:792-832    b2RayCastShape: cast in the shape's local frame
//   geometry.c:506-870 circle, capsule, segment and zero-radius polygon casts
//
// The trees only cull; the answer is the minimum-fraction hit over all shapes,
// found here by a linear scan. Equal fractions resolve to the lower shape id.
#include "port.h"

#include <stdlib.h>

#include <stddef.h>

World* p_world( int w ); // pworld.c

typedef struct CastOut
{
	v2 point, normal;
	float fraction;
	int hit;
} CastOut;

static CastOut cast_none( void )
{
	CastOut o;
	o.point = V( 0.0f, 0.0f );
	o.normal = V( 0.0f, 0.0f );
	o.fraction = 0.0f;
	o.hit = 0;
	return o;
}

// geometry.c:506-580
static CastOut ray_circle( v2 origin, v2 translation, float maxFraction, v2 center, float r )
{
	CastOut o = cast_none();
	v2 s = sub( origin, center );
	float rr = r * r;
	float len;
	v2 d = lengthAndNormalize( &len, translation );
	if ( len == 0.0f )
	{
		if ( lengthSq( s ) < rr )
		{
			o.point = origin;
			o.hit = 1;
		}
		return o;
	}
	float t = -dot( s, d );
	v2 c = mulAdd( s, t, d );
	float cc = dot( c, c );
	if ( cc > rr )
		return o;
	float h = sqrtf( rr - cc );
	float fraction = t - h;
	if ( fraction < 0.0f || maxFraction * len < fraction )
	{
		if ( lengthSq( s ) < rr )
		{
			o.point = origin;
			o.hit = 1;
		}
		return o;
	}
	v2 hp = mulAdd( s, fraction, d );
	o.fraction = fraction / len;
	o.normal = normalize( hp );
	o.point = mulAdd( center, r, o.normal );
	o.hit = 1;
	return o;
}

// geometry.c:582-716
static CastOut ray_capsule( v2 origin, v2 translation, float maxFraction, v2 v1, v2 v2p, float radius )
{
	CastOut o = cast_none();
	float capLen;
	v2 a = lengthAndNormalize( &capLen, sub( v2p, v1 ) );
	if ( capLen < FLT_EPSILON )
		return ray_circle( origin, translation, maxFraction, v1, radius );
	v2 q = sub( origin, v1 );
	float qa = dot( q, a );
	v2 qp = mulAdd( q, -qa, a );
	if ( dot( qp, qp ) < radius * radius )
	{
		// origin inside the capsule's rectangle band or one of its end caps
		if ( qa < 0.0f )
			return ray_circle( origin, translation, maxFraction, v1, radius );
		if ( qa > capLen )
			return ray_circle( origin, translation, maxFraction, v2p, radius );
		o.point = origin;
		o.hit = 1;
		return o;
	}
	v2 n = V( a.y, -a.x );
	float rayLen;
	v2 u = lengthAndNormalize( &rayLen, translation );
	float den = -a.x * u.y + u.x * a.y;
	if ( -FLT_EPSILON < den && den < FLT_EPSILON )
		return o;
	v2 b1 = mulSub( q, radius, n );
	v2 b2 = mulAdd( q, radius, n );
	float invDen = 1.0f / den;
	float s21 = ( a.x * b1.y - b1.x * a.y ) * invDen;
	float s22 = ( a.x * b2.y - b2.x * a.y ) * invDen;
	float s2;
	v2 b;
	if ( s21 < s22 )
	{
		s2 = s21;
		b = b1;
	}
	else
	{
		s2 = s22;
		b = b2;
		n = neg( n );
	}
	if ( s2 < 0.0f || maxFraction * rayLen < s2 )
		return o;
	float s1 = ( -b.x * u.y + u.x * b.y ) * invDen;
	if ( s1 < 0.0f )
		return ray_circle( origin, translation, maxFraction, v1, radius );
	if ( capLen < s1 )
		return ray_circle( origin, translation, maxFraction, v2p, radius );
	o.fraction = s2 / rayLen;
	o.point = add( lerp( v1, v2p, s1 / capLen ), mulSV( radius, n ) );
	o.normal = n;
	o.hit = 1;
	return o;
}

// geometry.c:718-797 (two-sided)
static CastOut ray_segment( v2 origin, v2 translation, float maxFraction, v2 v1, v2 v2p )
{
	CastOut o = cast_none();
	float len;
	v2 eu = lengthAndNormalize( &len, sub( v2p, v1 ) );
	if ( len == 0.0f )
		return o;
	v2 normal = rightPerp( eu );
	float num = dot( normal, sub( v1, origin ) );
	float den = dot( normal, translation );
	if ( den == 0.0f )
		return o;
	float t = num / den;
	if ( t < 0.0f || maxFraction < t )
		return o;
	v2 p = mulAdd( origin, t, translation );
	float s = dot( sub( p, v1 ), eu );
	if ( s < 0.0f || len < s )
		return o;
	if ( num > 0.0f )
		normal = neg( normal );
	o.fraction = t;
	o.point = p;
	o.normal = normal;
	o.hit = 1;
	return o;
}

// geometry.c:799-878, zero-radius branch
static CastOut ray_polygon( v2 origin, v2 d, float maxFraction, const Polygon* poly )
{
	CastOut o = cast_none();
	v2 base = poly->vertices[0];
	v2 p1 = sub( origin, base );
	float lower = 0.0f, upper = maxFraction;
	int index = -1;
	for ( int i = 0; i < poly->count; ++i )
	{
		v2 vertex = sub( poly->vertices[i], base );
		float num = dot( poly->normals[i], sub( vertex, p1 ) );
		float den = dot( poly->normals[i], d );
		if ( den == 0.0f )
		{
			if ( num < 0.0f )
				return o;
		}
		else if ( den < 0.0f && num < lower * den )
		{
			lower = num / den;
			index = i;
		}
		else if ( den > 0.0f && num < upper * den )
			upper = num / den;
		if ( upper < lower )
			return o;
	}
	if ( index >= 0 )
	{
		o.fraction = lower;
		o.normal = poly->normals[index];
		o.point = mulAdd( origin, lower, d );
	}
	else
		o.point = origin;
	o.hit = 1;
	return o;
}

// geometry.c:879-888 + distance.c:608-697 b2ShapeCast: a ray against a
// rounded polygon advances the origin conservatively on the GJK distance
// (radii off) until it is within the radius
static CastOut ray_rounded_polygon( v2 origin, v2 d, float maxFraction, const Polygon* poly )
{
	CastOut o = cast_none();
	ShapeProxy pa = p_make_proxy( poly->vertices, poly->count, poly->radius );
	ShapeProxy pb = p_make_proxy( &origin, 1, 0.0f );
	float target = fmaxp( P_LINEAR_SLOP, pa.radius + pb.radius - P_LINEAR_SLOP );
	float tolerance = 0.25f * P_LINEAR_SLOP;
	SimplexCache cache = { 0 };
	xform xfA = { { 0.0f, 0.0f }, { 1.0f, 0.0f } };
	xform xfB = xfA;
	float fraction = 0.0f;
	for ( int iteration = 0; iteration < 20; ++iteration )
	{
		v2 pA = V( 0.0f, 0.0f ), pB = V( 0.0f, 0.0f ), n = V( 0.0f, 0.0f );
		float dist = p_shape_distance( &pa, &pb, xfA, xfB, &cache, &pA, &pB, &n );
		if ( dist < target + tolerance )
		{
			o.hit = 1;
			if ( iteration == 0 )
			{
				// initial overlap: a common point
				v2 c1 = mulAdd( pA, pa.radius, n );
				v2 c2 = mulAdd( pB, -pb.radius, n );
				o.point = lerp( c1, c2, 0.5f );
				return o;
			}
			o.fraction = fraction;
			o.point = mulAdd( pA, pa.radius, n );
			o.normal = n;
			return o;
		}
		float den = dot( d, n );
		if ( den >= 0.0f )
			return o;
		fraction += ( target - dist ) / den;
		if ( fraction >= maxFraction )
			return o;
		xfB.p = mulAdd( V( 0.0f, 0.0f ), fraction, d );
	}
	return o;
}

static int query_collide( const Shape* s, uint64_t cat, uint64_t mask )
{
	return ( s->categoryBits & mask ) != 0 && ( s->maskBits & cat ) != 0;
}

// shape.c:792-832
static CastOut ray_shape( const Shape* s, xform xf, v2 origin, v2 translation )
{
	v2 lo = invXfPoint( xf, origin );
	v2 lt = invRotate( xf.q, translation );
	CastOut o;
	switch ( s->g.type )
	{
		case SHAPE_CIRCLE:
			o = ray_circle( lo, lt, 1.0f, s->g.c1, s->g.radius );
			break;
		case SHAPE_CAPSULE:
			o = ray_capsule( lo, lt, 1.0f, s->g.c1, s->g.c2, s->g.radius );
			break;
		case SHAPE_SEGMENT:
			o = ray_segment( lo, lt, 1.0f, s->g.c1, s->g.c2 );
			break;
		case SHAPE_CHAIN_SEGMENT:
			// geometry.c:718-729: one-sided, rays from the left side pass
			if ( cross( sub( lo, s->g.c1 ), sub( s->g.c2, s->g.c1 ) ) < 0.0f )
				return cast_none();
			o = ray_segment( lo, lt, 1.0f, s->g.c1, s->g.c2 );
			break;
		case SHAPE_POLYGON:
			if ( s->g.poly.radius != 0.0f )
				o = ray_rounded_polygon( lo, lt, 1.0f, &s->g.poly );
			else
				o = ray_polygon( lo, lt, 1.0f, &s->g.poly );
			break;
		default:
			return cast_none();
	}
	o.point = xfPoint( xf, o.point );
	o.normal = rotate( xf.q, o.normal );
	return o;
}

int orc_cast_ray_closest( int wi, double ox, double oy, double tx, double ty, long long cat, long long mask, int* shape,
						  float* out )
{
	World* w = p_world( wi );
	if ( w == NULL )
		return 0;
	v2 origin = V( (float)ox, (float)oy ), translation = V( (float)tx, (float)ty );
	int best = -1;
	CastOut bo = cast_none();
	for ( int i = 0; i < w->shapeCount; ++i )
	{
		const Shape* s = w->shapes + i;
		if ( s->used == 0 || s->proxyKey == P_NULL )
			continue;
		if ( query_collide( s, (uint64_t)cat, (uint64_t)mask ) == 0 )
			continue;
		CastOut o = ray_shape( s, w->bodies[s->bodyId].xf, origin, translation );
		if ( o.hit == 0 || o.fraction == 0.0f )
			continue;
		if ( best < 0 || o.fraction < bo.fraction )
		{
			best = i;
			bo = o;
		}
	}
	if ( best < 0 )
		return 0;
	*shape = best;
	out[0] = bo.point.x;
	out[1] = bo.point.y;
	out[2] = bo.normal.x;
	out[3] = bo.normal.y;
	out[4] = bo.fraction;
	return 1;
}

int orc_overlap_aabb( int wi, double lx, double ly, double ux, double uy, long long cat, long long mask, int* out,
					  int cap )
{
	World* w = p_world( wi );
	if ( w == NULL )
		return 0;
	box2 q;
	q.lo = V( (float)lx, (float)ly );
	q.hi = V( (float)ux, (float)uy );
	int n = 0;
	for ( int i = 0; i < w->shapeCount; ++i )
	{
		const Shape* s = w->shapes + i;
		if ( s->used == 0 || s->proxyKey == P_NULL )
			continue;
		if ( query_collide( s, (uint64_t)cat, (uint64_t)mask ) == 0 )
			continue;
		if ( boxOverlaps( s->fatAABB, q ) == false )
			continue;
		if ( n < cap )
			out[n] = i;
		n += 1;
	}
	return n;
}

// shape.c:655-703 b2GetShapeProjectedPerimeter
static float projected_perimeter( const Shape* s, v2 line )
{
	const Geometry* g = &s->g;
	switch ( g->type )
	{
		case SHAPE_CAPSULE:
		{
			v2 axis = sub( g->c2, g->c1 );
			float projectedLength = fabsp( dot( axis, line ) );
			return projectedLength + 2.0f * g->radius;
		}
		case SHAPE_CIRCLE:
			return 2.0f * g->radius;
		case SHAPE_POLYGON:
		{
			float value = dot( g->poly.vertices[0], line );
			float lower = value, upper = value;
			for ( int i = 1; i < g->poly.count; ++i )
			{
				value = dot( g->poly.vertices[i], line );
				lower = fminp( lower, value );
				upper = fmaxp( upper, value );
			}
			return ( upper - lower ) + 2.0f * g->poly.radius;
		}
		case SHAPE_SEGMENT:
		case SHAPE_CHAIN_SEGMENT:
		{
			float value1 = dot( g->c1, line );
			float value2 = dot( g->c2, line );
			return fabsp( value2 - value1 );
		}
		default:
			return 0.0f;
	}
}

// world.c:2640-2735 b2World_Explode: every shape of a dynamic body whose fat
// AABB meets the blast box (category against maskBits) and which lies within
// radius + falloff of the centre (GJK with radii) wakes its body and gets an
// impulse along the centre-to-closest-point direction, scaled by its
// projected perimeter and the falloff. Shapes are visited in id order (the
// reference visits its dynamic tree's order; the order only matters for a
// body with several shapes in the blast or for the order sleeping sets wake).
typedef struct ExplodeCtx
{
	World* w;
	v2 position;
	float r, fo, ipl;
} ExplodeCtx;

// world.c:2640-2716 ExplosionCallback, per shape in the dynamic tree's
// query order
static int explode_visit( int proxyId, int id, void* context )
{
	(void)proxyId;
	ExplodeCtx* e = context;
	World* w = e->w;
	const Shape* s = w->shapes + id;
	float r = e->r, fo = e->fo;
	v2 position = e->position;
	Body* b = w->bodies + s->bodyId;
	xform xf = b->xf;
	ShapeProxy pa = p_shape_proxy( &s->g );
	ShapeProxy pb = p_make_proxy( &position, 1, 0.0f );
	xform identity = { { 0.0f, 0.0f }, { 1.0f, 0.0f } };
	SimplexCache cache = { 0 };
	v2 pointA = V( 0.0f, 0.0f ), pointB = V( 0.0f, 0.0f ), normal = V( 0.0f, 0.0f );
	float d = p_shape_distance( &pa, &pb, xf, identity, &cache, &pointA, &pointB, &normal );
	// distance.c:592-603 useRadii
	if ( d > 0.1f * P_LINEAR_SLOP )
	{
		d = fmaxp( 0.0f, d - pa.radius - pb.radius );
		pointA = mulAdd( pointA, pa.radius, normal );
	}
	if ( d > r + fo )
		return 1;
	if ( b->setIndex >= SET_FIRST_SLEEPING )
		p_wake_solver_set( w, b->setIndex );
	if ( b->setIndex != SET_AWAKE )
		return 1;
	v2 closestPoint = pointA;
	if ( d == 0.0f )
		closestPoint = xfPoint( xf, p_shape_centroid( &s->g ) );
	v2 direction = sub( closestPoint, position );
	if ( lengthSq( direction ) > 100.0f * FLT_EPSILON * FLT_EPSILON )
		direction = normalize( direction );
	else
		direction = V( 1.0f, 0.0f );
	v2 localLine = invRotate( xf.q, leftPerp( direction ) );
	float perimeter = projected_perimeter( s, localLine );
	float scale = 1.0f;
	if ( d > r && fo > 0.0f )
		scale = fclampp( ( r + fo - d ) / fo, 0.0f, 1.0f );
	float magnitude = e->ipl * perimeter * scale;
	v2 impulse = mulSV( magnitude, direction );
	b->v = mulAdd( b->v, b->invMass, impulse );
	b->w += b->invInertia * cross( sub( closestPoint, b->center ), impulse );
	return 1;
}

// world.c:2718-2747 b2World_Explode: the dynamic tree's query over the
// blast box
void orc_world_explode( int wi, long long maskBits, double px, double py, double radius, double falloff,
						double impulsePerLength )
{
	World* w = p_world( wi );
	if ( w == NULL )
		return;
	ExplodeCtx e = { w, V( (float)px, (float)py ), (float)radius, (float)falloff, (float)impulsePerLength };
	box2 box;
	box.lo = V( e.position.x - ( e.r + e.fo ), e.position.y - ( e.r + e.fo ) );
	box.hi = V( e.position.x + ( e.r + e.fo ), e.position.y + ( e.r + e.fo ) );
	p_finish_tree_rebuild( w );
	rt_query( w->trees + BODY_DYNAMIC, box, (uint64_t)maskBits, explode_visit, &e );
}

typedef struct RayHitRow
{
	int shape;
	CastOut o;
} RayHitRow;

static int cmp_ray_hit( const void* a, const void* b )
{
	const RayHitRow* x = (const RayHitRow*)a;
	const RayHitRow* y = (const RayHitRow*)b;
	if ( x->o.fraction != y->o.fraction )
		return x->o.fraction < y->o.fraction ? -1 : 1;
	return x->shape < y->shape ? -1 : ( x->shape > y->shape ? 1 : 0 );
}

// world.c:2176-2251 b2World_CastRay with a callback: the hits of the whole
// ray are reported in ascending fraction (then shape id), the order in
// which a ray clipped by each returned fraction meets them; a hit beyond the
// current clip is not reported, 0 ends the cast, -1 skips the hit. (The
// reference reports in its trees' order; closest-hit, any-hit and all-hit
// callbacks end with the same answer.) Returns the number of calls.
int orc_world_cast_ray( int wi, double ox, double oy, double tx, double ty, long long cat, long long mask,
						orc_cast_fn fn, void* context )
{
	World* w = p_world( wi );
	if ( w == NULL || fn == NULL )
		return 0;
	v2 origin = V( (float)ox, (float)oy ), translation = V( (float)tx, (float)ty );
	RayHitRow* rows = (RayHitRow*)malloc( sizeof( RayHitRow ) * (size_t)( w->shapeCount > 0 ? w->shapeCount : 1 ) );
	int n = 0;
	for ( int i = 0; i < w->shapeCount; ++i )
	{
		const Shape* s = w->shapes + i;
		if ( s->used == 0 || s->proxyKey == P_NULL || query_collide( s, (uint64_t)cat, (uint64_t)mask ) == 0 )
			continue;
		CastOut o = ray_shape( s, w->bodies[s->bodyId].xf, origin, translation );
		if ( o.hit )
		{
			rows[n].shape = i;
			rows[n].o = o;
			n += 1;
		}
	}
	qsort( rows, (size_t)n, sizeof( RayHitRow ), cmp_ray_hit );
	float clip = 1.0f;
	int calls = 0;
	for ( int k = 0; k < n; ++k )
	{
		const CastOut* o = &rows[k].o;
		if ( o->fraction > clip )
			break;
		float r = fn( rows[k].shape, o->point.x, o->point.y, o->normal.x, o->normal.y, o->fraction, context );
		calls += 1;
		if ( r == 0.0f )
			break;
		if ( 0.0f <= r && r <= 1.0f )
			clip = r;
	}
	free( rows );
	return calls;
}
