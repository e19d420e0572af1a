// GJK distance and conservative-advancement time of impact of the
// restatement. TEST INFRASTRUCTURE (oracle). Reference:
// packages/forge2d/third_party/box2d/src/distance.c:9-25 (sweep transform),
// :99-112 (proxies), :138-560 (GJK simplex solver, b2ShapeDistance),
// :918-1096 (separation functions), :1137-1414 (b2TimeOfImpact).
#include "port.h"

#include <string.h>

typedef struct SimplexVertex
{
	v2 wA, wB, w;
	float a;
	int indexA, indexB;
} SimplexVertex;

typedef struct Simplex
{
	SimplexVertex v1, v2, v3;
	int count;
} Simplex;

static xform sweep_xf( const Sweep* s, float time )
{
	xform xf;
	xf.p = add( mulSV( 1.0f - time, s->c1 ), mulSV( time, s->c2 ) );
	rot q = { ( 1.0f - time ) * s->q1.c + time * s->q2.c, ( 1.0f - time ) * s->q1.s + time * s->q2.s };
	xf.q = normalizeRot( q );
	xf.p = sub( xf.p, rotate( xf.q, s->localCenter ) );
	return xf;
}

ShapeProxy p_make_proxy( const v2* pts, int count, float radius )
{
	ShapeProxy p;
	memset( &p, 0, sizeof( p ) );
	count = iminp( count, P_MAX_POLY );
	for ( int i = 0; i < count; ++i )
		p.points[i] = pts[i];
	p.count = count;
	p.radius = radius;
	return p;
}

// shape.c:922-943
ShapeProxy p_shape_proxy( const Geometry* g )
{
	v2 two[2] = { g->c1, g->c2 };
	switch ( g->type )
	{
		case SHAPE_CAPSULE:
			return p_make_proxy( two, 2, g->radius );
		case SHAPE_CIRCLE:
			return p_make_proxy( &g->c1, 1, g->radius );
		case SHAPE_POLYGON:
			return p_make_proxy( g->poly.vertices, g->poly.count, g->poly.radius );
		default:
			return p_make_proxy( two, 2, 0.0f );
	}
}

static int find_support( const ShapeProxy* p, v2 d )
{
	int best = 0;
	float bestValue = dot( p->points[0], d );
	for ( int i = 1; i < p->count; ++i )
	{
		float v = dot( p->points[i], d );
		if ( v > bestValue )
		{
			best = i;
			bestValue = v;
		}
	}
	return best;
}

static Simplex simplex_from_cache( const SimplexCache* cache, const ShapeProxy* pa, const ShapeProxy* pb )
{
	Simplex s;
	memset( &s, 0, sizeof( s ) );
	s.count = cache->count;
	SimplexVertex* vs[] = { &s.v1, &s.v2, &s.v3 };
	for ( int i = 0; i < s.count; ++i )
	{
		SimplexVertex* v = vs[i];
		v->indexA = cache->indexA[i];
		v->indexB = cache->indexB[i];
		v->wA = pa->points[v->indexA];
		v->wB = pb->points[v->indexB];
		v->w = sub( v->wA, v->wB );
		v->a = -1.0f;
	}
	if ( s.count == 0 )
	{
		SimplexVertex* v = vs[0];
		v->indexA = 0;
		v->indexB = 0;
		v->wA = pa->points[0];
		v->wB = pb->points[0];
		v->w = sub( v->wA, v->wB );
		v->a = 1.0f;
		s.count = 1;
	}
	return s;
}

static void witness( v2* a, v2* b, const Simplex* s )
{
	switch ( s->count )
	{
		case 1:
			*a = s->v1.wA;
			*b = s->v1.wB;
			break;
		case 2:
			*a = V( s->v1.a * s->v1.wA.x + s->v2.a * s->v2.wA.x, s->v1.a * s->v1.wA.y + s->v2.a * s->v2.wA.y );
			*b = V( s->v1.a * s->v1.wB.x + s->v2.a * s->v2.wB.x, s->v1.a * s->v1.wB.y + s->v2.a * s->v2.wB.y );
			break;
		case 3:
			*a = V( s->v1.a * s->v1.wA.x + s->v2.a * s->v2.wA.x + s->v3.a * s->v3.wA.x,
					s->v1.a * s->v1.wA.y + s->v2.a * s->v2.wA.y + s->v3.a * s->v3.wA.y );
			*b = *a;
			break;
		default:
			*a = V( 0.0f, 0.0f );
			*b = V( 0.0f, 0.0f );
			break;
	}
}

static v2 solve2( Simplex* s )
{
	v2 w1 = s->v1.w;
	v2 w2 = s->v2.w;
	v2 e12 = sub( w2, w1 );
	float d12_2 = -dot( w1, e12 );
	if ( d12_2 <= 0.0f )
	{
		s->v1.a = 1.0f;
		s->count = 1;
		return neg( w1 );
	}
	float d12_1 = dot( w2, e12 );
	if ( d12_1 <= 0.0f )
	{
		s->v2.a = 1.0f;
		s->count = 1;
		s->v1 = s->v2;
		return neg( w2 );
	}
	float inv_d12 = 1.0f / ( d12_1 + d12_2 );
	s->v1.a = d12_1 * inv_d12;
	s->v2.a = d12_2 * inv_d12;
	s->count = 2;
	return crossSV( cross( add( w1, w2 ), e12 ), e12 );
}

static v2 solve3( Simplex* s )
{
	v2 w1 = s->v1.w;
	v2 w2 = s->v2.w;
	v2 w3 = s->v3.w;
	v2 e12 = sub( w2, w1 );
	float w1e12 = dot( w1, e12 );
	float w2e12 = dot( w2, e12 );
	float d12_1 = w2e12;
	float d12_2 = -w1e12;
	v2 e13 = sub( w3, w1 );
	float w1e13 = dot( w1, e13 );
	float w3e13 = dot( w3, e13 );
	float d13_1 = w3e13;
	float d13_2 = -w1e13;
	v2 e23 = sub( w3, w2 );
	float w2e23 = dot( w2, e23 );
	float w3e23 = dot( w3, e23 );
	float d23_1 = w3e23;
	float d23_2 = -w2e23;
	float n123 = cross( e12, e13 );
	float d123_1 = n123 * cross( w2, w3 );
	float d123_2 = n123 * cross( w3, w1 );
	float d123_3 = n123 * cross( w1, w2 );
	if ( d12_2 <= 0.0f && d13_2 <= 0.0f )
	{
		s->v1.a = 1.0f;
		s->count = 1;
		return neg( w1 );
	}
	if ( d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f )
	{
		float inv = 1.0f / ( d12_1 + d12_2 );
		s->v1.a = d12_1 * inv;
		s->v2.a = d12_2 * inv;
		s->count = 2;
		return crossSV( cross( add( w1, w2 ), e12 ), e12 );
	}
	if ( d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f )
	{
		float inv = 1.0f / ( d13_1 + d13_2 );
		s->v1.a = d13_1 * inv;
		s->v3.a = d13_2 * inv;
		s->count = 2;
		s->v2 = s->v3;
		return crossSV( cross( add( w1, w3 ), e13 ), e13 );
	}
	if ( d12_1 <= 0.0f && d23_2 <= 0.0f )
	{
		s->v2.a = 1.0f;
		s->count = 1;
		s->v1 = s->v2;
		return neg( w2 );
	}
	if ( d13_1 <= 0.0f && d23_1 <= 0.0f )
	{
		s->v3.a = 1.0f;
		s->count = 1;
		s->v1 = s->v3;
		return neg( w3 );
	}
	if ( d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f )
	{
		float inv = 1.0f / ( d23_1 + d23_2 );
		s->v2.a = d23_1 * inv;
		s->v3.a = d23_2 * inv;
		s->count = 2;
		s->v1 = s->v3;
		return crossSV( cross( add( w2, w3 ), e23 ), e23 );
	}
	float inv = 1.0f / ( d123_1 + d123_2 + d123_3 );
	s->v1.a = d123_1 * inv;
	s->v2.a = d123_2 * inv;
	s->v3.a = d123_3 * inv;
	s->count = 3;
	return V( 0.0f, 0.0f );
}

// distance.c:421-606 b2ShapeDistance with useRadii = false: the distance,
// the witness points in the world frame of A (optional) and the updated
// cache (left alone when the shapes overlap)
float p_shape_distance( const ShapeProxy* pa, const ShapeProxy* pbIn, xform xfA, xform xfB, SimplexCache* cache,
						v2* pointA, v2* pointB, v2* normal )
{
	if ( normal != NULL )
		*normal = V( 0.0f, 0.0f );
	ShapeProxy pb;
	{
		xform t = invMulXf( xfA, xfB );
		pb.count = pbIn->count;
		pb.radius = pbIn->radius;
		for ( int i = 0; i < pb.count; ++i )
			pb.points[i] = xfPoint( t, pbIn->points[i] );
	}
	Simplex simplex = simplex_from_cache( cache, pa, &pb );
	SimplexVertex* vs[] = { &simplex.v1, &simplex.v2, &simplex.v3 };
	v2 nonUnitNormal = V( 0.0f, 0.0f );
	int saveA[3], saveB[3];
	const int maxIterations = 20;
	int iteration = 0;
	while ( iteration < maxIterations )
	{
		int saveCount = simplex.count;
		for ( int i = 0; i < saveCount; ++i )
		{
			saveA[i] = vs[i]->indexA;
			saveB[i] = vs[i]->indexB;
		}
		v2 d = V( 0.0f, 0.0f );
		switch ( simplex.count )
		{
			case 1:
				d = neg( simplex.v1.w );
				break;
			case 2:
				d = solve2( &simplex );
				break;
			case 3:
				d = solve3( &simplex );
				break;
			default:
				break;
		}
		if ( simplex.count == 3 || dot( d, d ) < FLT_EPSILON * FLT_EPSILON )
		{
			if ( pointA != NULL )
			{
				v2 la, lb;
				witness( &la, &lb, &simplex );
				*pointA = xfPoint( xfA, la );
				*pointB = xfPoint( xfA, lb );
			}
			return 0.0f;
		}
		nonUnitNormal = d;
		SimplexVertex* vertex = vs[simplex.count];
		vertex->indexA = find_support( pa, d );
		vertex->wA = pa->points[vertex->indexA];
		vertex->indexB = find_support( &pb, neg( d ) );
		vertex->wB = pb.points[vertex->indexB];
		vertex->w = sub( vertex->wA, vertex->wB );
		++iteration;
		bool duplicate = false;
		for ( int i = 0; i < saveCount; ++i )
		{
			if ( vertex->indexA == saveA[i] && vertex->indexB == saveB[i] )
			{
				duplicate = true;
				break;
			}
		}
		if ( duplicate )
			break;
		simplex.count += 1;
	}
	if ( normal != NULL )
		*normal = rotate( xfA.q, normalize( nonUnitNormal ) );
	v2 la, lb;
	witness( &la, &lb, &simplex );
	float dx = lb.x - la.x;
	float dy = lb.y - la.y;
	float distance = sqrtf( dx * dx + dy * dy );
	if ( pointA != NULL )
	{
		*pointA = xfPoint( xfA, la );
		*pointB = xfPoint( xfA, lb );
	}
	cache->count = simplex.count;
	for ( int i = 0; i < simplex.count; ++i )
	{
		cache->indexA[i] = (uint8_t)vs[i]->indexA;
		cache->indexB[i] = (uint8_t)vs[i]->indexB;
	}
	return distance;
}

enum
{
	SEP_POINTS = 0,
	SEP_FACE_A = 1,
	SEP_FACE_B = 2,
};

typedef struct SepFn
{
	const ShapeProxy* pa;
	const ShapeProxy* pb;
	Sweep sa, sb;
	v2 localPoint;
	v2 axis;
	int type;
} SepFn;

static SepFn make_sep( const SimplexCache* cache, const ShapeProxy* pa, const Sweep* sa, const ShapeProxy* pb,
					   const Sweep* sb, float t1 )
{
	SepFn f;
	f.pa = pa;
	f.pb = pb;
	int count = cache->count;
	f.sa = *sa;
	f.sb = *sb;
	xform xfA = sweep_xf( sa, t1 );
	xform xfB = sweep_xf( sb, t1 );
	if ( count == 1 )
	{
		f.type = SEP_POINTS;
		v2 pA = xfPoint( xfA, pa->points[cache->indexA[0]] );
		v2 pB = xfPoint( xfB, pb->points[cache->indexB[0]] );
		f.axis = normalize( sub( pB, pA ) );
		f.localPoint = V( 0.0f, 0.0f );
		return f;
	}
	if ( cache->indexA[0] == cache->indexA[1] )
	{
		f.type = SEP_FACE_B;
		v2 b1 = pb->points[cache->indexB[0]];
		v2 b2 = pb->points[cache->indexB[1]];
		f.axis = crossVS( sub( b2, b1 ), 1.0f );
		f.axis = normalize( f.axis );
		v2 normal = rotate( xfB.q, f.axis );
		f.localPoint = V( 0.5f * ( b1.x + b2.x ), 0.5f * ( b1.y + b2.y ) );
		v2 pB = xfPoint( xfB, f.localPoint );
		v2 pA = xfPoint( xfA, pa->points[cache->indexA[0]] );
		float s = dot( sub( pA, pB ), normal );
		if ( s < 0.0f )
			f.axis = neg( f.axis );
		return f;
	}
	f.type = SEP_FACE_A;
	v2 a1 = pa->points[cache->indexA[0]];
	v2 a2 = pa->points[cache->indexA[1]];
	f.axis = crossVS( sub( a2, a1 ), 1.0f );
	f.axis = normalize( f.axis );
	v2 normal = rotate( xfA.q, f.axis );
	f.localPoint = V( 0.5f * ( a1.x + a2.x ), 0.5f * ( a1.y + a2.y ) );
	v2 pA = xfPoint( xfA, f.localPoint );
	v2 pB = xfPoint( xfB, pb->points[cache->indexB[0]] );
	float s = dot( sub( pB, pA ), normal );
	if ( s < 0.0f )
		f.axis = neg( f.axis );
	return f;
}

static float find_min_sep( const SepFn* f, int* ia, int* ib, float t )
{
	xform xfA = sweep_xf( &f->sa, t );
	xform xfB = sweep_xf( &f->sb, t );
	switch ( f->type )
	{
		case SEP_POINTS:
		{
			v2 axisA = invRotate( xfA.q, f->axis );
			v2 axisB = invRotate( xfB.q, neg( f->axis ) );
			*ia = find_support( f->pa, axisA );
			*ib = find_support( f->pb, axisB );
			v2 pA = xfPoint( xfA, f->pa->points[*ia] );
			v2 pB = xfPoint( xfB, f->pb->points[*ib] );
			return dot( sub( pB, pA ), f->axis );
		}
		case SEP_FACE_A:
		{
			v2 normal = rotate( xfA.q, f->axis );
			v2 pA = xfPoint( xfA, f->localPoint );
			v2 axisB = invRotate( xfB.q, neg( normal ) );
			*ia = -1;
			*ib = find_support( f->pb, axisB );
			v2 pB = xfPoint( xfB, f->pb->points[*ib] );
			return dot( sub( pB, pA ), normal );
		}
		default:
		{
			v2 normal = rotate( xfB.q, f->axis );
			v2 pB = xfPoint( xfB, f->localPoint );
			v2 axisA = invRotate( xfA.q, neg( normal ) );
			*ib = -1;
			*ia = find_support( f->pa, axisA );
			v2 pA = xfPoint( xfA, f->pa->points[*ia] );
			return dot( sub( pA, pB ), normal );
		}
	}
}

static float eval_sep( const SepFn* f, int ia, int ib, float t )
{
	xform xfA = sweep_xf( &f->sa, t );
	xform xfB = sweep_xf( &f->sb, t );
	switch ( f->type )
	{
		case SEP_POINTS:
		{
			v2 pA = xfPoint( xfA, f->pa->points[ia] );
			v2 pB = xfPoint( xfB, f->pb->points[ib] );
			return dot( sub( pB, pA ), f->axis );
		}
		case SEP_FACE_A:
		{
			v2 normal = rotate( xfA.q, f->axis );
			v2 pA = xfPoint( xfA, f->localPoint );
			v2 pB = xfPoint( xfB, f->pb->points[ib] );
			return dot( sub( pB, pA ), normal );
		}
		default:
		{
			v2 normal = rotate( xfB.q, f->axis );
			v2 pB = xfPoint( xfB, f->localPoint );
			v2 pA = xfPoint( xfA, f->pa->points[ia] );
			return dot( sub( pA, pB ), normal );
		}
	}
}

// distance.c:1137-1414; *state receives 0 unknown, 1 failed, 2 overlapped,
// 3 hit, 4 separated (b2TOIState order)
float p_time_of_impact( const ShapeProxy* pa, const ShapeProxy* pb, Sweep sa, Sweep sb, float tMax, int* state )
{
	*state = 0;
	float fraction = tMax;
	float totalRadius = pa->radius + pb->radius;
	float target = fmaxp( P_LINEAR_SLOP, totalRadius - P_LINEAR_SLOP );
	float tolerance = 0.25f * P_LINEAR_SLOP;
	float t1 = 0.0f;
	const int kMax = 20;
	int distanceIterations = 0;
	SimplexCache cache;
	memset( &cache, 0, sizeof( cache ) );
	for ( ;; )
	{
		xform xfA = sweep_xf( &sa, t1 );
		xform xfB = sweep_xf( &sb, t1 );
		float distance = p_shape_distance( pa, pb, xfA, xfB, &cache, NULL, NULL, NULL );
		distanceIterations += 1;
		if ( distance <= 0.0f )
		{
			*state = 2;
			fraction = 0.0f;
			break;
		}
		if ( distance <= target + tolerance )
		{
			*state = 3;
			fraction = t1;
			break;
		}
		SepFn fcn = make_sep( &cache, pa, &sa, pb, &sb, t1 );
		bool done = false;
		float t2 = tMax;
		int pushBackIterations = 0;
		for ( ;; )
		{
			int ia, ib;
			float s2 = find_min_sep( &fcn, &ia, &ib, t2 );
			if ( s2 > target + tolerance )
			{
				*state = 4;
				fraction = tMax;
				done = true;
				break;
			}
			if ( s2 > target - tolerance )
			{
				t1 = t2;
				break;
			}
			float s1 = eval_sep( &fcn, ia, ib, t1 );
			if ( s1 < target - tolerance )
			{
				*state = 1;
				fraction = t1;
				done = true;
				break;
			}
			if ( s1 <= target + tolerance )
			{
				*state = 3;
				fraction = t1;
				done = true;
				break;
			}
			int rootIterationCount = 0;
			float a1 = t1, a2 = t2;
			for ( ;; )
			{
				float t;
				if ( rootIterationCount & 1 )
					t = a1 + ( target - s1 ) * ( a2 - a1 ) / ( s2 - s1 );
				else
					t = 0.5f * ( a1 + a2 );
				rootIterationCount += 1;
				float s = eval_sep( &fcn, ia, ib, t );
				if ( fabsp( s - target ) < tolerance )
				{
					t2 = t;
					break;
				}
				if ( s > target )
				{
					a1 = t;
					s1 = s;
				}
				else
				{
					a2 = t;
					s2 = s;
				}
				if ( rootIterationCount == 50 )
					break;
			}
			pushBackIterations += 1;
			if ( pushBackIterations == P_MAX_POLY )
				break;
		}
		if ( done )
			break;
		if ( distanceIterations == kMax )
		{
			*state = 1;
			fraction = t1;
			break;
		}
	}
	return fraction;
}
