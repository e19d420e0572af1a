// Device GJK distance and conservative-advancement time of impact for
// continuous collision. Same computation and operand order as Box2D v3.1.1
// packages/forge2d/third_party/box2d/src/distance.c:9-25 (sweep transform),
// :138-560 (GJK), :918-1096 (separation functions), :1137-1414
// (b2TimeOfImpact).
#pragma once

#include "dmath.cuh"

struct DProxy
{
	fv2 p[F2D_MAX_POLY];
	int count;
	float radius;
};

struct DSweep
{
	fv2 localCenter;
	fv2 c1, c2;
	frot q1, q2;
};

struct DSimplexVertex
{
	fv2 wA, wB, w;
	float a;
	int indexA, indexB;
};

struct DSimplex
{
	DSimplexVertex v[3];
	int count;
};

struct DCache
{
	int count;
	int indexA[3];
	int indexB[3];
};

__device__ __forceinline__ fxf sweep_xf( const DSweep& s, float t )
{
	fxf xf;
	xf.p = vadd( vscale( 1.0f - t, s.c1 ), vscale( t, s.c2 ) );
	frot q;
	q.c = ( 1.0f - t ) * s.q1.c + t * s.q2.c;
	q.s = ( 1.0f - t ) * s.q1.s + t * s.q2.s;
	xf.q = rnormalize( q );
	xf.p = vsub( xf.p, rrot( xf.q, s.localCenter ) );
	return xf;
}

__device__ __forceinline__ int support( const DProxy& p, fv2 d )
{
	int best = 0;
	float bv = vdot( p.p[0], d );
	for ( int i = 1; i < p.count; ++i )
	{
		float v = vdot( p.p[i], d );
		if ( v > bv )
		{
			best = i;
			bv = v;
		}
	}
	return best;
}

__device__ __forceinline__ fv2 solve2( DSimplex& s )
{
	fv2 w1 = s.v[0].w, w2 = s.v[1].w;
	fv2 e12 = vsub( w2, w1 );
	float d12_2 = -vdot( w1, e12 );
	if ( d12_2 <= 0.0f )
	{
		s.v[0].a = 1.0f;
		s.count = 1;
		return vneg( w1 );
	}
	float d12_1 = vdot( w2, e12 );
	if ( d12_1 <= 0.0f )
	{
		s.v[1].a = 1.0f;
		s.count = 1;
		s.v[0] = s.v[1];
		return vneg( w2 );
	}
	float inv = 1.0f / ( d12_1 + d12_2 );
	s.v[0].a = d12_1 * inv;
	s.v[1].a = d12_2 * inv;
	s.count = 2;
	return vcrossSV( vcross( vadd( w1, w2 ), e12 ), e12 );
}

__device__ __forceinline__ fv2 solve3( DSimplex& s )
{
	fv2 w1 = s.v[0].w, w2 = s.v[1].w, w3 = s.v[2].w;
	fv2 e12 = vsub( w2, w1 );
	float w1e12 = vdot( w1, e12 ), w2e12 = vdot( w2, e12 );
	float d12_1 = w2e12, d12_2 = -w1e12;
	fv2 e13 = vsub( w3, w1 );
	float w1e13 = vdot( w1, e13 ), w3e13 = vdot( w3, e13 );
	float d13_1 = w3e13, d13_2 = -w1e13;
	fv2 e23 = vsub( w3, w2 );
	float w2e23 = vdot( w2, e23 ), w3e23 = vdot( w3, e23 );
	float d23_1 = w3e23, d23_2 = -w2e23;
	float n123 = vcross( e12, e13 );
	float d123_1 = n123 * vcross( w2, w3 );
	float d123_2 = n123 * vcross( w3, w1 );
	float d123_3 = n123 * vcross( w1, w2 );
	if ( d12_2 <= 0.0f && d13_2 <= 0.0f )
	{
		s.v[0].a = 1.0f;
		s.count = 1;
		return vneg( w1 );
	}
	if ( d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f )
	{
		float inv = 1.0f / ( d12_1 + d12_2 );
		s.v[0].a = d12_1 * inv;
		s.v[1].a = d12_2 * inv;
		s.count = 2;
		return vcrossSV( vcross( vadd( w1, w2 ), e12 ), e12 );
	}
	if ( d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f )
	{
		float inv = 1.0f / ( d13_1 + d13_2 );
		s.v[0].a = d13_1 * inv;
		s.v[2].a = d13_2 * inv;
		s.count = 2;
		s.v[1] = s.v[2];
		return vcrossSV( vcross( vadd( w1, w3 ), e13 ), e13 );
	}
	if ( d12_1 <= 0.0f && d23_2 <= 0.0f )
	{
		s.v[1].a = 1.0f;
		s.count = 1;
		s.v[0] = s.v[1];
		return vneg( w2 );
	}
	if ( d13_1 <= 0.0f && d23_1 <= 0.0f )
	{
		s.v[2].a = 1.0f;
		s.count = 1;
		s.v[0] = s.v[2];
		return vneg( w3 );
	}
	if ( d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f )
	{
		float inv = 1.0f / ( d23_1 + d23_2 );
		s.v[1].a = d23_1 * inv;
		s.v[2].a = d23_2 * inv;
		s.count = 2;
		s.v[0] = s.v[2];
		return vcrossSV( vcross( vadd( w2, w3 ), e23 ), e23 );
	}
	float inv = 1.0f / ( d123_1 + d123_2 + d123_3 );
	s.v[0].a = d123_1 * inv;
	s.v[1].a = d123_2 * inv;
	s.v[2].a = d123_3 * inv;
	s.count = 3;
	return mk( 0.0f, 0.0f );
}

__device__ __forceinline__ void gjk_witness( const DSimplex& s, fv2& la, fv2& lb )
{
	if ( s.count == 1 )
	{
		la = s.v[0].wA;
		lb = s.v[0].wB;
	}
	else if ( s.count == 2 )
	{
		la = mk( s.v[0].a * s.v[0].wA.x + s.v[1].a * s.v[1].wA.x, s.v[0].a * s.v[0].wA.y + s.v[1].a * s.v[1].wA.y );
		lb = mk( s.v[0].a * s.v[0].wB.x + s.v[1].a * s.v[1].wB.x, s.v[0].a * s.v[0].wB.y + s.v[1].a * s.v[1].wB.y );
	}
	else
	{
		la = mk( s.v[0].a * s.v[0].wA.x + s.v[1].a * s.v[1].wA.x + s.v[2].a * s.v[2].wA.x,
				 s.v[0].a * s.v[0].wA.y + s.v[1].a * s.v[1].wA.y + s.v[2].a * s.v[2].wA.y );
		lb = la;
	}
}

// b2ShapeDistance with useRadii = false (distance.c:421-606): returns the
// distance, updates the cache (left alone when the shapes overlap) and, when
// asked, gives the witness points in the world frame of A
static __device__ float gjk_distance( const DProxy& pa, const DProxy& pbIn, fxf xfA, fxf xfB, DCache& cache,
									  fv2* pointA = nullptr, fv2* pointB = nullptr, fv2* normalOut = nullptr )
{
	fv2 nonUnitNormal = mk( 0.0f, 0.0f );
	if ( normalOut != nullptr )
		*normalOut = nonUnitNormal;
	DProxy pb;
	{
		fxf t = xinvmul( xfA, xfB );
		pb.count = pbIn.count;
		pb.radius = pbIn.radius;
		for ( int i = 0; i < pb.count; ++i )
			pb.p[i] = xpoint( t, pbIn.p[i] );
	}
	DSimplex s;
	s.count = cache.count;
	for ( int i = 0; i < s.count; ++i )
	{
		s.v[i].indexA = cache.indexA[i];
		s.v[i].indexB = cache.indexB[i];
		s.v[i].wA = pa.p[s.v[i].indexA];
		s.v[i].wB = pb.p[s.v[i].indexB];
		s.v[i].w = vsub( s.v[i].wA, s.v[i].wB );
		s.v[i].a = -1.0f;
	}
	if ( s.count == 0 )
	{
		s.v[0].indexA = 0;
		s.v[0].indexB = 0;
		s.v[0].wA = pa.p[0];
		s.v[0].wB = pb.p[0];
		s.v[0].w = vsub( s.v[0].wA, s.v[0].wB );
		s.v[0].a = 1.0f;
		s.count = 1;
	}
	int saveA[3], saveB[3];
	int iteration = 0;
	while ( iteration < 20 )
	{
		int saveCount = s.count;
		for ( int i = 0; i < saveCount; ++i )
		{
			saveA[i] = s.v[i].indexA;
			saveB[i] = s.v[i].indexB;
		}
		fv2 d = mk( 0.0f, 0.0f );
		if ( s.count == 1 )
			d = vneg( s.v[0].w );
		else if ( s.count == 2 )
			d = solve2( s );
		else if ( s.count == 3 )
			d = solve3( s );
		if ( s.count == 3 || vdot( d, d ) < FLT_EPSILON * FLT_EPSILON )
		{
			if ( pointA != nullptr )
			{
				fv2 la, lb;
				gjk_witness( s, la, lb );
				*pointA = xpoint( xfA, la );
				*pointB = xpoint( xfA, lb );
			}
			return 0.0f;
		}
		nonUnitNormal = d;
		DSimplexVertex& vx = s.v[s.count];
		vx.indexA = support( pa, d );
		vx.wA = pa.p[vx.indexA];
		vx.indexB = support( pb, vneg( d ) );
		vx.wB = pb.p[vx.indexB];
		vx.w = vsub( vx.wA, vx.wB );
		++iteration;
		bool duplicate = false;
		for ( int i = 0; i < saveCount; ++i )
			if ( vx.indexA == saveA[i] && vx.indexB == saveB[i] )
			{
				duplicate = true;
				break;
			}
		if ( duplicate )
			break;
		s.count += 1;
	}
	if ( normalOut != nullptr )
		*normalOut = rrot( xfA.q, vnormalize( nonUnitNormal ) );
	fv2 la, lb;
	gjk_witness( s, la, lb );
	float dx = lb.x - la.x, dy = lb.y - la.y;
	float distance = sqrtf( dx * dx + dy * dy );
	if ( pointA != nullptr )
	{
		*pointA = xpoint( xfA, la );
		*pointB = xpoint( xfA, lb );
	}
	cache.count = s.count;
	for ( int i = 0; i < s.count; ++i )
	{
		cache.indexA[i] = s.v[i].indexA;
		cache.indexB[i] = s.v[i].indexB;
	}
	return distance;
}

struct DSep
{
	fv2 localPoint;
	fv2 axis;
	int type; // 0 points, 1 face A, 2 face B
};

__device__ __forceinline__ DSep make_sep( const DCache& cache, const DProxy& pa, const DSweep& sa, const DProxy& pb,
										  const DSweep& sb, float t1 )
{
	DSep f;
	fxf xfA = sweep_xf( sa, t1 );
	fxf xfB = sweep_xf( sb, t1 );
	if ( cache.count == 1 )
	{
		f.type = 0;
		fv2 pA = xpoint( xfA, pa.p[cache.indexA[0]] );
		fv2 pB = xpoint( xfB, pb.p[cache.indexB[0]] );
		f.axis = vnormalize( vsub( pB, pA ) );
		f.localPoint = mk( 0.0f, 0.0f );
		return f;
	}
	if ( cache.indexA[0] == cache.indexA[1] )
	{
		f.type = 2;
		fv2 b1 = pb.p[cache.indexB[0]];
		fv2 b2 = pb.p[cache.indexB[1]];
		f.axis = vcrossVS( vsub( b2, b1 ), 1.0f );
		f.axis = vnormalize( f.axis );
		fv2 normal = rrot( xfB.q, f.axis );
		f.localPoint = mk( 0.5f * ( b1.x + b2.x ), 0.5f * ( b1.y + b2.y ) );
		fv2 pB = xpoint( xfB, f.localPoint );
		fv2 pA = xpoint( xfA, pa.p[cache.indexA[0]] );
		float s = vdot( vsub( pA, pB ), normal );
		if ( s < 0.0f )
			f.axis = vneg( f.axis );
		return f;
	}
	f.type = 1;
	fv2 a1 = pa.p[cache.indexA[0]];
	fv2 a2 = pa.p[cache.indexA[1]];
	f.axis = vcrossVS( vsub( a2, a1 ), 1.0f );
	f.axis = vnormalize( f.axis );
	fv2 normal = rrot( xfA.q, f.axis );
	f.localPoint = mk( 0.5f * ( a1.x + a2.x ), 0.5f * ( a1.y + a2.y ) );
	fv2 pA = xpoint( xfA, f.localPoint );
	fv2 pB = xpoint( xfB, pb.p[cache.indexB[0]] );
	float s = vdot( vsub( pB, pA ), normal );
	if ( s < 0.0f )
		f.axis = vneg( f.axis );
	return f;
}

__device__ __forceinline__ float min_sep( const DSep& f, const DProxy& pa, const DSweep& sa, const DProxy& pb,
										  const DSweep& sb, int* ia, int* ib, float t )
{
	fxf xfA = sweep_xf( sa, t );
	fxf xfB = sweep_xf( sb, t );
	if ( f.type == 0 )
	{
		fv2 axisA = rinvrot( xfA.q, f.axis );
		fv2 axisB = rinvrot( xfB.q, vneg( f.axis ) );
		*ia = support( pa, axisA );
		*ib = support( pb, axisB );
		fv2 pA = xpoint( xfA, pa.p[*ia] );
		fv2 pB = xpoint( xfB, pb.p[*ib] );
		return vdot( vsub( pB, pA ), f.axis );
	}
	if ( f.type == 1 )
	{
		fv2 normal = rrot( xfA.q, f.axis );
		fv2 pA = xpoint( xfA, f.localPoint );
		fv2 axisB = rinvrot( xfB.q, vneg( normal ) );
		*ia = -1;
		*ib = support( pb, axisB );
		fv2 pB = xpoint( xfB, pb.p[*ib] );
		return vdot( vsub( pB, pA ), normal );
	}
	fv2 normal = rrot( xfB.q, f.axis );
	fv2 pB = xpoint( xfB, f.localPoint );
	fv2 axisA = rinvrot( xfA.q, vneg( normal ) );
	*ib = -1;
	*ia = support( pa, axisA );
	fv2 pA = xpoint( xfA, pa.p[*ia] );
	return vdot( vsub( pA, pB ), normal );
}

__device__ __forceinline__ float eval_sep( const DSep& f, const DProxy& pa, const DSweep& sa, const DProxy& pb,
										   const DSweep& sb, int ia, int ib, float t )
{
	fxf xfA = sweep_xf( sa, t );
	fxf xfB = sweep_xf( sb, t );
	if ( f.type == 0 )
	{
		fv2 pA = xpoint( xfA, pa.p[ia] );
		fv2 pB = xpoint( xfB, pb.p[ib] );
		return vdot( vsub( pB, pA ), f.axis );
	}
	if ( f.type == 1 )
	{
		fv2 normal = rrot( xfA.q, f.axis );
		fv2 pA = xpoint( xfA, f.localPoint );
		fv2 pB = xpoint( xfB, pb.p[ib] );
		return vdot( vsub( pB, pA ), normal );
	}
	fv2 normal = rrot( xfB.q, f.axis );
	fv2 pB = xpoint( xfB, f.localPoint );
	fv2 pA = xpoint( xfA, pa.p[ia] );
	return vdot( vsub( pA, pB ), normal );
}

static __device__ float time_of_impact( const DProxy& pa, const DProxy& pb, const DSweep& sa, const DSweep& sb, float tMax )
{
	float fraction = tMax;
	float totalRadius = pa.radius + pb.radius;
	float target = fmax_s( F2D_LINEAR_SLOP, totalRadius - F2D_LINEAR_SLOP );
	float tolerance = 0.25f * F2D_LINEAR_SLOP;
	float t1 = 0.0f;
	int distanceIterations = 0;
	DCache cache;
	cache.count = 0;
	for ( ;; )
	{
		fxf xfA = sweep_xf( sa, t1 );
		fxf xfB = sweep_xf( sb, t1 );
		float distance = gjk_distance( pa, pb, xfA, xfB, cache );
		distanceIterations += 1;
		if ( distance <= 0.0f )
		{
			fraction = 0.0f;
			break;
		}
		if ( distance <= target + tolerance )
		{
			fraction = t1;
			break;
		}
		DSep fcn = make_sep( cache, pa, sa, pb, sb, t1 );
		bool done = false;
		float t2 = tMax;
		int pushBackIterations = 0;
		for ( ;; )
		{
			int ia, ib;
			float s2 = min_sep( fcn, pa, sa, pb, sb, &ia, &ib, t2 );
			if ( s2 > target + tolerance )
			{
				fraction = tMax;
				done = true;
				break;
			}
			if ( s2 > target - tolerance )
			{
				t1 = t2;
				break;
			}
			float s1 = eval_sep( fcn, pa, sa, pb, sb, ia, ib, t1 );
			if ( s1 < target - tolerance )
			{
				fraction = t1;
				done = true;
				break;
			}
			if ( s1 <= target + tolerance )
			{
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
				float s = eval_sep( fcn, pa, sa, pb, sb, ia, ib, t );
				if ( fabs_s( s - target ) < tolerance )
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
			if ( pushBackIterations == F2D_MAX_POLY )
				break;
		}
		if ( done )
			break;
		if ( distanceIterations == 20 )
		{
			fraction = t1;
			break;
		}
	}
	return fraction;
}
