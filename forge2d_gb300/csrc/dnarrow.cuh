// Device narrowphase: contact manifolds for circle, capsule, segment and
// convex-polygon pairs. Each function computes what the corresponding
// b2Collide* of Box2D v3.1.1 computes (packages/forge2d/third_party/box2d/
// src/manifold.c, cited per function), with the same operand order so the
// results are bit-identical under -fmad=false.
#pragma once

#include "dmath.cuh"
#include "dtoi.cuh"
#include "dworld.cuh"

#define MAKE_ID( A, B ) ( (unsigned)( ( ( (unsigned)(A)&0xffu ) << 8 ) | ( (unsigned)(B)&0xffu ) ) )

struct DPoly
{
	fv2 v[F2D_MAX_POLY];
	fv2 n[F2D_MAX_POLY];
	float radius;
	int count;
};

struct DGeom
{
	int type;
	fv2 c1, c2;
	float radius;
	DPoly poly;
	fv2 g1, g2; // chain segment ghost vertices
};

struct DPoint
{
	fv2 anchorA, anchorB, point;
	float separation;
	unsigned id;
};

struct DManifold
{
	fv2 normal;
	DPoint p[2];
	int count;
};

// Every manifold starts zeroed, like the reference's `b2Manifold manifold =
// { 0 }`: a slot past pointCount then holds exactly what the manifold
// function left there (b2CollidePolygons' vertex-vertex fallback keeps the
// second clip point), and the stored manifold reproduces it.
__device__ __forceinline__ DManifold dm_empty()
{
	DManifold m;
	m.normal = mk( 0.0f, 0.0f );
	for ( int k = 0; k < 2; ++k )
	{
		m.p[k].anchorA = mk( 0.0f, 0.0f );
		m.p[k].anchorB = mk( 0.0f, 0.0f );
		m.p[k].point = mk( 0.0f, 0.0f );
		m.p[k].separation = 0.0f;
		m.p[k].id = 0u;
	}
	m.count = 0;
	return m;
}

__device__ __forceinline__ DGeom load_geom( const float4* __restrict__ g, int type )
{
	DGeom o;
	o.type = type;
	float4 g0 = g[0];
	float4 g1 = g[1];
	o.c1 = mk( g0.x, g0.y );
	o.c2 = mk( g0.z, g0.w );
	o.radius = g1.x;
	o.poly.radius = g1.x;
	o.poly.count = __float_as_int( g1.y );
	if ( type == ST_CHAIN )
	{
		float4 gh = g[2];
		o.g1 = mk( gh.x, gh.y );
		o.g2 = mk( gh.z, gh.w );
	}
	if ( type == 3 )
	{
#pragma unroll
		for ( int i = 0; i < 4; ++i )
		{
			float4 a = g[2 + i];
			float4 b = g[6 + i];
			o.poly.v[2 * i] = mk( a.x, a.y );
			o.poly.v[2 * i + 1] = mk( a.z, a.w );
			o.poly.n[2 * i] = mk( b.x, b.y );
			o.poly.n[2 * i + 1] = mk( b.z, b.w );
		}
	}
	return o;
}

// distance.c:27-97 (b2SegmentDistance)
struct DSegDist
{
	fv2 c1, c2;
	float f1, f2, dist2;
};

__device__ __forceinline__ DSegDist seg_distance( fv2 p1, fv2 q1, fv2 p2, fv2 q2 )
{
	DSegDist r;
	fv2 d1 = vsub( q1, p1 );
	fv2 d2 = vsub( q2, p2 );
	fv2 rr = vsub( p1, p2 );
	float dd1 = vdot( d1, d1 );
	float dd2 = vdot( d2, d2 );
	float rd1 = vdot( rr, d1 );
	float rd2 = vdot( rr, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	if ( dd1 < epsSqr || dd2 < epsSqr )
	{
		if ( dd1 >= epsSqr )
		{
			r.f1 = fclamp_s( -rd1 / dd1, 0.0f, 1.0f );
			r.f2 = 0.0f;
		}
		else if ( dd2 >= epsSqr )
		{
			r.f1 = 0.0f;
			r.f2 = fclamp_s( rd2 / dd2, 0.0f, 1.0f );
		}
		else
		{
			r.f1 = 0.0f;
			r.f2 = 0.0f;
		}
	}
	else
	{
		float d12 = vdot( d1, d2 );
		float denom = dd1 * dd2 - d12 * d12;
		float f1 = 0.0f;
		if ( denom != 0.0f )
			f1 = fclamp_s( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
		float f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2 < 0.0f )
		{
			f2 = 0.0f;
			f1 = fclamp_s( -rd1 / dd1, 0.0f, 1.0f );
		}
		else if ( f2 > 1.0f )
		{
			f2 = 1.0f;
			f1 = fclamp_s( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
		}
		r.f1 = f1;
		r.f2 = f2;
	}
	r.c1 = vmuladd( p1, r.f1, d1 );
	r.c2 = vmuladd( p2, r.f2, d2 );
	r.dist2 = vdist2( r.c1, r.c2 );
	return r;
}

__device__ __forceinline__ void one_point( DManifold& m, fxf xfA, fxf xfB, fv2 cpA, float sep, unsigned id )
{
	m.p[0].anchorA = rrot( xfA.q, cpA );
	m.p[0].anchorB = vadd( m.p[0].anchorA, vsub( xfA.p, xfB.p ) );
	m.p[0].point = vadd( xfA.p, m.p[0].anchorA );
	m.p[0].separation = sep;
	m.p[0].id = id;
	m.count = 1;
}

// manifold.c:40-75 (b2CollideCircles)
__device__ __forceinline__ DManifold collide_circles( fv2 cA, float rA, fxf xfA, fv2 cB, float rB, fxf xfB )
{
	DManifold m = dm_empty();
	fxf xf = xinvmul( xfA, xfB );
	fv2 pointA = cA;
	fv2 pointB = xpoint( xf, cB );
	float distance;
	fv2 normal = vlen_norm( &distance, vsub( pointB, pointA ) );
	float separation = distance - rA - rB;
	if ( separation > F2D_SPECULATIVE )
		return m;
	fv2 ca = vmuladd( pointA, rA, normal );
	fv2 cb = vmuladd( pointB, -rB, normal );
	fv2 cp = vlerp( ca, cb, 0.5f );
	m.normal = rrot( xfA.q, normal );
	one_point( m, xfA, xfB, cp, separation, 0 );
	return m;
}

// manifold.c:77-139 (b2CollideCapsuleAndCircle)
__device__ __forceinline__ DManifold collide_capsule_circle( fv2 p1, fv2 p2, float rA, fxf xfA, fv2 cB, float rB,
															 fxf xfB )
{
	DManifold m = dm_empty();
	fxf xf = xinvmul( xfA, xfB );
	fv2 pB = xpoint( xf, cB );
	fv2 e = vsub( p2, p1 );
	fv2 pA;
	float s1 = vdot( vsub( pB, p1 ), e );
	float s2 = vdot( vsub( p2, pB ), e );
	if ( s1 < 0.0f )
		pA = p1;
	else if ( s2 < 0.0f )
		pA = p2;
	else
	{
		float s = s1 / vdot( e, e );
		pA = vmuladd( p1, s, e );
	}
	float distance;
	fv2 normal = vlen_norm( &distance, vsub( pB, pA ) );
	float separation = distance - rA - rB;
	if ( separation > F2D_SPECULATIVE )
		return m;
	fv2 ca = vmuladd( pA, rA, normal );
	fv2 cb = vmuladd( pB, -rB, normal );
	fv2 cp = vlerp( ca, cb, 0.5f );
	m.normal = rrot( xfA.q, normal );
	one_point( m, xfA, xfB, cp, separation, 0 );
	return m;
}

// manifold.c:141-259 (b2CollidePolygonAndCircle)
__device__ __forceinline__ DManifold collide_polygon_circle( const DPoly& pa, fxf xfA, fv2 cB, float rB, fxf xfB )
{
	DManifold m = dm_empty();
	fxf xf = xinvmul( xfA, xfB );
	fv2 center = xpoint( xf, cB );
	float rA = pa.radius;
	float radius = rA + rB;
	int normalIndex = 0;
	float separation = -FLT_MAX;
	for ( int i = 0; i < pa.count; ++i )
	{
		float s = vdot( pa.n[i], vsub( center, pa.v[i] ) );
		if ( s > separation )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation > radius + F2D_SPECULATIVE )
		return m;
	int i1 = normalIndex;
	int i2 = i1 + 1 < pa.count ? i1 + 1 : 0;
	fv2 v1 = pa.v[i1];
	fv2 v2 = pa.v[i2];
	float u1 = vdot( vsub( center, v1 ), vsub( v2, v1 ) );
	float u2 = vdot( vsub( center, v2 ), vsub( v1, v2 ) );
	if ( u1 < 0.0f && separation > FLT_EPSILON )
	{
		fv2 normal = vnormalize( vsub( center, v1 ) );
		separation = vdot( vsub( center, v1 ), normal );
		if ( separation > radius + F2D_SPECULATIVE )
			return m;
		fv2 ca = vmuladd( v1, rA, normal );
		fv2 cb = vmulsub( center, rB, normal );
		fv2 cp = vlerp( ca, cb, 0.5f );
		m.normal = rrot( xfA.q, normal );
		one_point( m, xfA, xfB, cp, vdot( vsub( cb, ca ), normal ), 0 );
	}
	else if ( u2 < 0.0f && separation > FLT_EPSILON )
	{
		fv2 normal = vnormalize( vsub( center, v2 ) );
		separation = vdot( vsub( center, v2 ), normal );
		if ( separation > radius + F2D_SPECULATIVE )
			return m;
		fv2 ca = vmuladd( v2, rA, normal );
		fv2 cb = vmulsub( center, rB, normal );
		fv2 cp = vlerp( ca, cb, 0.5f );
		m.normal = rrot( xfA.q, normal );
		one_point( m, xfA, xfB, cp, vdot( vsub( cb, ca ), normal ), 0 );
	}
	else
	{
		fv2 normal = pa.n[normalIndex];
		m.normal = rrot( xfA.q, normal );
		fv2 ca = vmuladd( center, rA - vdot( vsub( center, v1 ), normal ), normal );
		fv2 cb = vmulsub( center, rB, normal );
		fv2 cp = vlerp( ca, cb, 0.5f );
		one_point( m, xfA, xfB, cp, separation - radius, 0 );
	}
	return m;
}

// manifold.c:261-530 (b2CollideCapsules; segments use radius 0)
static __device__ __noinline__ DManifold collide_capsules( fv2 a1, fv2 a2, float rA, fxf xfA, fv2 b1, fv2 b2, float rB, fxf xfB )
{
	fv2 origin = a1;
	fxf sfA;
	sfA.p = vadd( xfA.p, rrot( xfA.q, origin ) );
	sfA.q = xfA.q;
	fxf xf = xinvmul( sfA, xfB );
	fv2 p1 = mk( 0.0f, 0.0f );
	fv2 q1 = vsub( a2, origin );
	fv2 p2 = xpoint( xf, b1 );
	fv2 q2 = xpoint( xf, b2 );
	fv2 d1 = vsub( q1, p1 );
	fv2 d2 = vsub( q2, p2 );
	float dd1 = vdot( d1, d1 );
	float dd2 = vdot( d2, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	fv2 r = vsub( p1, p2 );
	float rd1 = vdot( r, d1 );
	float rd2 = vdot( r, d2 );
	float d12 = vdot( d1, d2 );
	float denom = dd1 * dd2 - d12 * d12;
	float f1 = 0.0f;
	if ( denom != 0.0f )
		f1 = fclamp_s( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
	float f2 = ( d12 * f1 + rd2 ) / dd2;
	if ( f2 < 0.0f )
	{
		f2 = 0.0f;
		f1 = fclamp_s( -rd1 / dd1, 0.0f, 1.0f );
	}
	else if ( f2 > 1.0f )
	{
		f2 = 1.0f;
		f1 = fclamp_s( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
	}
	fv2 closest1 = vmuladd( p1, f1, d1 );
	fv2 closest2 = vmuladd( p2, f2, d2 );
	float distanceSquared = vdist2( closest1, closest2 );
	DManifold m = dm_empty();
	float radius = rA + rB;
	float maxDistance = radius + F2D_SPECULATIVE;
	if ( distanceSquared > maxDistance * maxDistance )
		return m;
	float distance = sqrtf( distanceSquared );
	float length1, length2;
	fv2 u1 = vlen_norm( &length1, d1 );
	fv2 u2 = vlen_norm( &length2, d2 );
	float fp2 = vdot( vsub( p2, p1 ), u1 );
	float fq2 = vdot( vsub( q2, p1 ), u1 );
	bool outsideA = ( fp2 <= 0.0f && fq2 <= 0.0f ) || ( fp2 >= length1 && fq2 >= length1 );
	float fp1 = vdot( vsub( p1, p2 ), u2 );
	float fq1 = vdot( vsub( q1, p2 ), u2 );
	bool outsideB = ( fp1 <= 0.0f && fq1 <= 0.0f ) || ( fp1 >= length2 && fq1 >= length2 );
	if ( outsideA == false && outsideB == false )
	{
		fv2 normalA;
		float separationA;
		{
			normalA = vleft( u1 );
			float ss1 = vdot( vsub( p2, p1 ), normalA );
			float ss2 = vdot( vsub( q2, p1 ), normalA );
			float s1p = ss1 < ss2 ? ss1 : ss2;
			float s1n = -ss1 < -ss2 ? -ss1 : -ss2;
			if ( s1p > s1n )
				separationA = s1p;
			else
			{
				separationA = s1n;
				normalA = vneg( normalA );
			}
		}
		fv2 normalB;
		float separationB;
		{
			normalB = vleft( u2 );
			float ss1 = vdot( vsub( p1, p2 ), normalB );
			float ss2 = vdot( vsub( q1, p2 ), normalB );
			float s1p = ss1 < ss2 ? ss1 : ss2;
			float s1n = -ss1 < -ss2 ? -ss1 : -ss2;
			if ( s1p > s1n )
				separationB = s1p;
			else
			{
				separationB = s1n;
				normalB = vneg( normalB );
			}
		}
		if ( separationA + 0.1f * F2D_LINEAR_SLOP >= separationB )
		{
			m.normal = normalA;
			fv2 cp = p2;
			fv2 cq = q2;
			if ( fp2 < 0.0f && fq2 > 0.0f )
				cp = vlerp( p2, q2, ( 0.0f - fp2 ) / ( fq2 - fp2 ) );
			else if ( fq2 < 0.0f && fp2 > 0.0f )
				cq = vlerp( q2, p2, ( 0.0f - fq2 ) / ( fp2 - fq2 ) );
			if ( fp2 > length1 && fq2 < length1 )
				cp = vlerp( p2, q2, ( fp2 - length1 ) / ( fp2 - fq2 ) );
			else if ( fq2 > length1 && fp2 < length1 )
				cq = vlerp( q2, p2, ( fq2 - length1 ) / ( fq2 - fp2 ) );
			float sp = vdot( vsub( cp, p1 ), normalA );
			float sq = vdot( vsub( cq, p1 ), normalA );
			if ( sp <= distance + F2D_LINEAR_SLOP || sq <= distance + F2D_LINEAR_SLOP )
			{
				m.p[0].anchorA = vmuladd( cp, 0.5f * ( rA - rB - sp ), normalA );
				m.p[0].separation = sp - radius;
				m.p[0].id = MAKE_ID( 0, 0 );
				m.p[1].anchorA = vmuladd( cq, 0.5f * ( rA - rB - sq ), normalA );
				m.p[1].separation = sq - radius;
				m.p[1].id = MAKE_ID( 0, 1 );
				m.count = 2;
			}
		}
		else
		{
			m.normal = vneg( normalB );
			fv2 cp = p1;
			fv2 cq = q1;
			if ( fp1 < 0.0f && fq1 > 0.0f )
				cp = vlerp( p1, q1, ( 0.0f - fp1 ) / ( fq1 - fp1 ) );
			else if ( fq1 < 0.0f && fp1 > 0.0f )
				cq = vlerp( q1, p1, ( 0.0f - fq1 ) / ( fp1 - fq1 ) );
			if ( fp1 > length2 && fq1 < length2 )
				cp = vlerp( p1, q1, ( fp1 - length2 ) / ( fp1 - fq1 ) );
			else if ( fq1 > length2 && fp1 < length2 )
				cq = vlerp( q1, p1, ( fq1 - length2 ) / ( fq1 - fp1 ) );
			float sp = vdot( vsub( cp, p2 ), normalB );
			float sq = vdot( vsub( cq, p2 ), normalB );
			if ( sp <= distance + F2D_LINEAR_SLOP || sq <= distance + F2D_LINEAR_SLOP )
			{
				m.p[0].anchorA = vmuladd( cp, 0.5f * ( rB - rA - sp ), normalB );
				m.p[0].separation = sp - radius;
				m.p[0].id = MAKE_ID( 0, 0 );
				m.p[1].anchorA = vmuladd( cq, 0.5f * ( rB - rA - sq ), normalB );
				m.p[1].separation = sq - radius;
				m.p[1].id = MAKE_ID( 1, 0 );
				m.count = 2;
			}
		}
	}
	if ( m.count == 0 )
	{
		fv2 normal = vsub( closest2, closest1 );
		if ( vdot( normal, normal ) > epsSqr )
			normal = vnormalize( normal );
		else
			normal = vleft( u1 );
		fv2 c1 = vmuladd( closest1, rA, normal );
		fv2 c2 = vmuladd( closest2, -rB, normal );
		int i1 = f1 == 0.0f ? 0 : 1;
		int i2 = f2 == 0.0f ? 0 : 1;
		m.normal = normal;
		m.p[0].anchorA = vlerp( c1, c2, 0.5f );
		m.p[0].separation = sqrtf( distanceSquared ) - radius;
		m.p[0].id = MAKE_ID( i1, i2 );
		m.count = 1;
	}
	m.normal = rrot( xfA.q, m.normal );
	for ( int i = 0; i < m.count; ++i )
	{
		m.p[i].anchorA = rrot( xfA.q, vadd( m.p[i].anchorA, origin ) );
		m.p[i].anchorB = vadd( m.p[i].anchorA, vsub( xfA.p, xfB.p ) );
		m.p[i].point = vadd( xfA.p, m.p[i].anchorA );
	}
	return m;
}

// manifold.c:16-34: a capsule as a 2-gon
__device__ __forceinline__ void capsule_poly( DPoly& s, fv2 p1, fv2 p2, float radius )
{
	s.v[0] = p1;
	s.v[1] = p2;
	fv2 axis = vnormalize( vsub( p2, p1 ) );
	fv2 n = vright( axis );
	s.n[0] = n;
	s.n[1] = vneg( n );
	s.count = 2;
	s.radius = radius;
}

// manifold.c:680-718 (b2FindMaxSeparation)
__device__ __forceinline__ float find_max_sep( int* edge, const DPoly& p1, const DPoly& p2 )
{
	int best = 0;
	float maxSep = -FLT_MAX;
	for ( int i = 0; i < p1.count; ++i )
	{
		fv2 n = p1.n[i];
		fv2 v1 = p1.v[i];
		float si = FLT_MAX;
		for ( int j = 0; j < p2.count; ++j )
		{
			float sij = vdot( n, vsub( p2.v[j], v1 ) );
			if ( sij < si )
				si = sij;
		}
		if ( si > maxSep )
		{
			maxSep = si;
			best = i;
		}
	}
	*edge = best;
	return maxSep;
}

// manifold.c:545-678 (b2ClipPolygons)
__device__ __forceinline__ DManifold clip_polygons( const DPoly& pA, const DPoly& pB, int edgeA, int edgeB, bool flip )
{
	DManifold m = dm_empty();
	const DPoly& poly1 = flip ? pB : pA;
	const DPoly& poly2 = flip ? pA : pB;
	int i11, i12, i21, i22;
	if ( flip )
	{
		i11 = edgeB;
		i12 = edgeB + 1 < pB.count ? edgeB + 1 : 0;
		i21 = edgeA;
		i22 = edgeA + 1 < pA.count ? edgeA + 1 : 0;
	}
	else
	{
		i11 = edgeA;
		i12 = edgeA + 1 < pA.count ? edgeA + 1 : 0;
		i21 = edgeB;
		i22 = edgeB + 1 < pB.count ? edgeB + 1 : 0;
	}
	fv2 normal = poly1.n[i11];
	fv2 v11 = poly1.v[i11];
	fv2 v12 = poly1.v[i12];
	fv2 v21 = poly2.v[i21];
	fv2 v22 = poly2.v[i22];
	fv2 tangent = vcrossSV( 1.0f, normal );
	float lower1 = 0.0f;
	float upper1 = vdot( vsub( v12, v11 ), tangent );
	float upper2 = vdot( vsub( v21, v11 ), tangent );
	float lower2 = vdot( vsub( v22, v11 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 )
		return m;
	fv2 vLower;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON )
		vLower = vlerp( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = v22;
	fv2 vUpper;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON )
		vUpper = vlerp( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = v21;
	float sepLower = vdot( vsub( vLower, v11 ), normal );
	float sepUpper = vdot( vsub( vUpper, v11 ), normal );
	float r1 = poly1.radius;
	float r2 = poly2.radius;
	vLower = vmuladd( vLower, 0.5f * ( r1 - r2 - sepLower ), normal );
	vUpper = vmuladd( vUpper, 0.5f * ( r1 - r2 - sepUpper ), normal );
	float radius = r1 + r2;
	if ( flip == false )
	{
		m.normal = normal;
		m.p[0].anchorA = vLower;
		m.p[0].separation = sepLower - radius;
		m.p[0].id = MAKE_ID( i11, i22 );
		m.p[1].anchorA = vUpper;
		m.p[1].separation = sepUpper - radius;
		m.p[1].id = MAKE_ID( i12, i21 );
	}
	else
	{
		m.normal = vneg( normal );
		m.p[0].anchorA = vUpper;
		m.p[0].separation = sepUpper - radius;
		m.p[0].id = MAKE_ID( i21, i12 );
		m.p[1].anchorA = vLower;
		m.p[1].separation = sepLower - radius;
		m.p[1].id = MAKE_ID( i22, i11 );
	}
	m.count = 2;
	return m;
}

__device__ __forceinline__ void vertex_vertex( DManifold& m, fv2 va, fv2 vb, float ra, float rb, float distance,
											   float radius, unsigned id )
{
	fv2 normal = vsub( vb, va );
	float invDistance = 1.0f / distance;
	normal.x *= invDistance;
	normal.y *= invDistance;
	fv2 c1 = vmuladd( va, ra, normal );
	fv2 c2 = vmuladd( vb, -rb, normal );
	m.normal = normal;
	m.p[0].anchorA = vlerp( c1, c2, 0.5f );
	m.p[0].separation = distance - radius;
	m.p[0].id = id;
	m.count = 1;
}

// manifold.c:736-1075 (b2CollidePolygons)
static __device__ __noinline__ DManifold collide_polygons( const DPoly& polygonA, fxf xfA, const DPoly& polygonB, fxf xfB )
{
	fv2 origin = polygonA.v[0];
	fxf sfA;
	sfA.p = vadd( xfA.p, rrot( xfA.q, origin ) );
	sfA.q = xfA.q;
	fxf xf = xinvmul( sfA, xfB );
	DPoly la;
	la.count = polygonA.count;
	la.radius = polygonA.radius;
	la.v[0] = mk( 0.0f, 0.0f );
	la.n[0] = polygonA.n[0];
	for ( int i = 1; i < la.count; ++i )
	{
		la.v[i] = vsub( polygonA.v[i], origin );
		la.n[i] = polygonA.n[i];
	}
	DPoly lb;
	lb.count = polygonB.count;
	lb.radius = polygonB.radius;
	for ( int i = 0; i < lb.count; ++i )
	{
		lb.v[i] = xpoint( xf, polygonB.v[i] );
		lb.n[i] = rrot( xf.q, polygonB.n[i] );
	}
	int edgeA = 0;
	float separationA = find_max_sep( &edgeA, la, lb );
	int edgeB = 0;
	float separationB = find_max_sep( &edgeB, lb, la );
	float radius = la.radius + lb.radius;
	DManifold m = dm_empty();
	if ( separationA > F2D_SPECULATIVE + radius || separationB > F2D_SPECULATIVE + radius )
		return m;
	bool flip;
	if ( separationA >= separationB )
	{
		flip = false;
		fv2 sd = la.n[edgeA];
		edgeB = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < lb.count; ++i )
		{
			float d = vdot( sd, lb.n[i] );
			if ( d < minDot )
			{
				minDot = d;
				edgeB = i;
			}
		}
	}
	else
	{
		flip = true;
		fv2 sd = lb.n[edgeB];
		edgeA = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < la.count; ++i )
		{
			float d = vdot( sd, la.n[i] );
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}
	if ( separationA > 0.1f * F2D_LINEAR_SLOP || separationB > 0.1f * F2D_LINEAR_SLOP )
	{
		int i11 = edgeA;
		int i12 = edgeA + 1 < la.count ? edgeA + 1 : 0;
		int i21 = edgeB;
		int i22 = edgeB + 1 < lb.count ? edgeB + 1 : 0;
		fv2 v11 = la.v[i11];
		fv2 v12 = la.v[i12];
		fv2 v21 = lb.v[i21];
		fv2 v22 = lb.v[i22];
		DSegDist res = seg_distance( v11, v12, v21, v22 );
		float distance = sqrtf( res.dist2 );
		float separation = distance - radius;
		if ( distance - radius > F2D_SPECULATIVE )
			return m;
		m = clip_polygons( la, lb, edgeA, edgeB, flip );
		float minSeparation = FLT_MAX;
		for ( int i = 0; i < m.count; ++i )
			minSeparation = fmin_s( minSeparation, m.p[i].separation );
		if ( separation + 0.1f * F2D_LINEAR_SLOP < minSeparation )
		{
			if ( res.f1 == 0.0f && res.f2 == 0.0f )
				vertex_vertex( m, v11, v21, la.radius, lb.radius, distance, radius, MAKE_ID( i11, i21 ) );
			else if ( res.f1 == 0.0f && res.f2 == 1.0f )
				vertex_vertex( m, v11, v22, la.radius, lb.radius, distance, radius, MAKE_ID( i11, i22 ) );
			else if ( res.f1 == 1.0f && res.f2 == 0.0f )
				vertex_vertex( m, v12, v21, la.radius, lb.radius, distance, radius, MAKE_ID( i12, i21 ) );
			else if ( res.f1 == 1.0f && res.f2 == 1.0f )
				vertex_vertex( m, v12, v22, la.radius, lb.radius, distance, radius, MAKE_ID( i12, i22 ) );
		}
	}
	else
	{
		m = clip_polygons( la, lb, edgeA, edgeB, flip );
	}
	if ( m.count > 0 )
	{
		m.normal = rrot( xfA.q, m.normal );
		for ( int i = 0; i < m.count; ++i )
		{
			m.p[i].anchorA = rrot( xfA.q, vadd( m.p[i].anchorA, origin ) );
			m.p[i].anchorB = vadd( m.p[i].anchorA, vsub( xfA.p, xfB.p ) );
			m.p[i].point = vadd( xfA.p, m.p[i].anchorA );
		}
	}
	return m;
}

// manifold.c:1089-1168 b2CollideChainSegmentAndCircle: one-sided, with the
// ghost vertices' Voronoi regions
__device__ __forceinline__ DManifold collide_chain_circle( const DGeom& a, fxf xfA, fv2 cB, float radius, fxf xfB )
{
	DManifold m = dm_empty();
	fxf xf = xinvmul( xfA, xfB );
	fv2 pB = xpoint( xf, cB );
	fv2 p1 = a.c1, p2 = a.c2;
	fv2 e = vsub( p2, p1 );
	float offset = vdot( vright( e ), vsub( pB, p1 ) );
	if ( offset < 0.0f )
		return m;
	float u = vdot( e, vsub( p2, pB ) );
	float v = vdot( e, vsub( pB, p1 ) );
	fv2 pA;
	if ( v <= 0.0f )
	{
		fv2 prevEdge = vsub( p1, a.g1 );
		float uPrev = vdot( prevEdge, vsub( pB, p1 ) );
		if ( uPrev <= 0.0f )
			return m;
		pA = p1;
	}
	else if ( u <= 0.0f )
	{
		fv2 nextEdge = vsub( a.g2, p2 );
		float vNext = vdot( nextEdge, vsub( pB, p2 ) );
		if ( vNext > 0.0f )
			return m;
		pA = p2;
	}
	else
	{
		float ee = vdot( e, e );
		pA = mk( u * p1.x + v * p2.x, u * p1.y + v * p2.y );
		pA = ee > 0.0f ? vscale( 1.0f / ee, pA ) : p1;
	}
	float distance;
	fv2 normal = vlen_norm( &distance, vsub( pB, pA ) );
	float separation = distance - radius;
	if ( separation > F2D_SPECULATIVE )
		return m;
	fv2 cA = pA;
	fv2 cb = vmuladd( pB, -radius, normal );
	fv2 cp = vlerp( cA, cb, 0.5f );
	m.normal = rrot( xfA.q, normal );
	one_point( m, xfA, xfB, cp, separation, 0 );
	return m;
}

// manifold.c:1177-1254 b2ClipSegments (frame of the segment, unrotated)
__device__ __forceinline__ DManifold clip_segments( fv2 a1, fv2 a2, fv2 b1, fv2 b2, fv2 normal, float ra, float rb,
													unsigned id1, unsigned id2 )
{
	DManifold m = dm_empty();
	fv2 tangent = vleft( normal );
	float lower1 = 0.0f;
	float upper1 = vdot( vsub( a2, a1 ), tangent );
	float upper2 = vdot( vsub( b1, a1 ), tangent );
	float lower2 = vdot( vsub( b2, a1 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 )
		return m;
	fv2 vLower;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON )
		vLower = vlerp( b2, b1, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = b2;
	fv2 vUpper;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON )
		vUpper = vlerp( b2, b1, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = b1;
	float separationLower = vdot( vsub( vLower, a1 ), normal );
	float separationUpper = vdot( vsub( vUpper, a1 ), normal );
	vLower = vmuladd( vLower, 0.5f * ( ra - rb - separationLower ), normal );
	vUpper = vmuladd( vUpper, 0.5f * ( ra - rb - separationUpper ), normal );
	float radius = ra + rb;
	m.normal = normal;
	m.p[0].anchorA = vLower;
	m.p[0].separation = separationLower - radius;
	m.p[0].id = id1;
	m.p[1].anchorA = vUpper;
	m.p[1].separation = separationUpper - radius;
	m.p[1].id = id2;
	m.count = 2;
	return m;
}

#define NORMAL_SKIP 0
#define NORMAL_ADMIT 1
#define NORMAL_SNAP 2

struct DChainParams
{
	fv2 edge1, normal0, normal2;
	bool convex1, convex2;
};

// manifold.c:1270-1316 b2ClassifyNormal
__device__ __forceinline__ int classify_normal( const DChainParams& p, fv2 normal )
{
	const float sinTol = 0.01f;
	if ( vdot( normal, p.edge1 ) <= 0.0f )
	{
		if ( p.convex1 )
			return vcross( normal, p.normal0 ) > sinTol ? NORMAL_SKIP : NORMAL_ADMIT;
		return NORMAL_SNAP;
	}
	if ( p.convex2 )
		return vcross( p.normal2, normal ) > sinTol ? NORMAL_SKIP : NORMAL_ADMIT;
	return NORMAL_SNAP;
}

__device__ __forceinline__ void finish_clip( DManifold& m, fxf xfA, fxf xfB, fv2 normalLocal )
{
	if ( m.count != 2 )
		return;
	m.normal = rrot( xfA.q, normalLocal );
	m.p[0].anchorA = rrot( xfA.q, m.p[0].anchorA );
	m.p[1].anchorA = rrot( xfA.q, m.p[1].anchorA );
	fv2 pAB = vsub( xfA.p, xfB.p );
	m.p[0].anchorB = vadd( m.p[0].anchorA, pAB );
	m.p[1].anchorB = vadd( m.p[1].anchorA, pAB );
	m.p[0].point = vadd( xfA.p, m.p[0].anchorA );
	m.p[1].point = vadd( xfA.p, m.p[1].anchorA );
}

// manifold.c:1318-1726 b2CollideChainSegmentAndPolygon: GJK warm-started from
// the contact's simplex cache selects vertex-vertex, vertex-edge or the SAT
// over the segment normal, its convex neighbours and the admitted polygon
// normals; the Gauss map of the chain vertices skips or snaps ghost normals
static __device__ DManifold collide_chain_polygon( const DGeom& a, fxf xfA, const DPoly& polygonB, fv2 polygonCentroid,
										   fxf xfB, DCache& cache )
{
	DManifold m = dm_empty();
	fxf xf = xinvmul( xfA, xfB );
	fv2 centroidB = xpoint( xf, polygonCentroid );
	float radiusB = polygonB.radius;
	fv2 p1 = a.c1, p2 = a.c2;
	fv2 edge1 = vnormalize( vsub( p2, p1 ) );
	DChainParams sp;
	sp.edge1 = edge1;
	const float convexTol = 0.01f;
	fv2 edge0 = vnormalize( vsub( p1, a.g1 ) );
	sp.normal0 = vright( edge0 );
	sp.convex1 = vcross( edge0, edge1 ) >= convexTol;
	fv2 edge2 = vnormalize( vsub( a.g2, p2 ) );
	sp.normal2 = vright( edge2 );
	sp.convex2 = vcross( edge1, edge2 ) >= convexTol;
	fv2 normal1 = vright( edge1 );
	bool behind1 = vdot( normal1, vsub( centroidB, p1 ) ) < 0.0f;
	bool behind0 = true, behind2 = true;
	if ( sp.convex1 )
		behind0 = vdot( sp.normal0, vsub( centroidB, p1 ) ) < 0.0f;
	if ( sp.convex2 )
		behind2 = vdot( sp.normal2, vsub( centroidB, p2 ) ) < 0.0f;
	if ( behind1 && behind0 && behind2 )
		return m;
	int count = polygonB.count;
	fv2 vertices[F2D_MAX_POLY];
	fv2 normals[F2D_MAX_POLY];
	for ( int i = 0; i < count; ++i )
	{
		vertices[i] = xpoint( xf, polygonB.v[i] );
		normals[i] = rrot( xf.q, polygonB.n[i] );
	}
	DProxy proxyA, proxyB;
	proxyA.p[0] = p1;
	proxyA.p[1] = p2;
	proxyA.count = 2;
	proxyA.radius = 0.0f;
	for ( int i = 0; i < count; ++i )
		proxyB.p[i] = vertices[i];
	proxyB.count = count;
	proxyB.radius = 0.0f;
	fxf identity;
	identity.p = mk( 0.0f, 0.0f );
	identity.q.c = 1.0f;
	identity.q.s = 0.0f;
	fv2 pointA = mk( 0.0f, 0.0f ), pointB = mk( 0.0f, 0.0f );
	float distance = gjk_distance( proxyA, proxyB, identity, identity, cache, &pointA, &pointB );
	if ( distance > radiusB + F2D_SPECULATIVE )
		return m;
	fv2 n0 = sp.convex1 ? sp.normal0 : normal1;
	fv2 n2 = sp.convex2 ? sp.normal2 : normal1;
	int incidentIndex = -1;
	int incidentNormal = -1;
	if ( behind1 == false && distance > 0.1f * F2D_LINEAR_SLOP )
	{
		if ( cache.count == 1 )
		{
			fv2 normal = vnormalize( vsub( pointB, pointA ) );
			int type = classify_normal( sp, normal );
			if ( type == NORMAL_SKIP )
				return m;
			if ( type == NORMAL_ADMIT )
			{
				m.normal = rrot( xfA.q, normal );
				m.p[0].anchorA = rrot( xfA.q, pointA );
				m.p[0].anchorB = vadd( m.p[0].anchorA, vsub( xfA.p, xfB.p ) );
				m.p[0].point = vadd( xfA.p, m.p[0].anchorA );
				m.p[0].separation = distance - radiusB;
				m.p[0].id = MAKE_ID( cache.indexA[0], cache.indexB[0] );
				m.count = 1;
				return m;
			}
			incidentIndex = cache.indexB[0];
		}
		else
		{
			int ia1 = cache.indexA[0];
			int ia2 = cache.indexA[1];
			int ib1 = cache.indexB[0];
			int ib2 = cache.indexB[1];
			if ( ia1 == ia2 )
			{
				fv2 normalB = vsub( pointA, pointB );
				float dot1 = vdot( normalB, normals[ib1] );
				float dot2 = vdot( normalB, normals[ib2] );
				int ib = dot1 > dot2 ? ib1 : ib2;
				normalB = normals[ib];
				int type = classify_normal( sp, vneg( normalB ) );
				if ( type == NORMAL_SKIP )
					return m;
				if ( type == NORMAL_ADMIT )
				{
					ib1 = ib;
					ib2 = ib < count - 1 ? ib + 1 : 0;
					fv2 b1 = vertices[ib1];
					fv2 b2 = vertices[ib2];
					dot1 = vdot( normalB, vsub( p1, b1 ) );
					dot2 = vdot( normalB, vsub( p2, b1 ) );
					if ( dot1 < dot2 )
					{
						if ( vdot( n0, normalB ) < vdot( normal1, normalB ) )
							return m;
					}
					else
					{
						if ( vdot( n2, normalB ) < vdot( normal1, normalB ) )
							return m;
					}
					m = clip_segments( b1, b2, p1, p2, normalB, radiusB, 0.0f, MAKE_ID( ib1, 1 ), MAKE_ID( ib2, 0 ) );
					finish_clip( m, xfA, xfB, vneg( normalB ) );
					return m;
				}
				incidentNormal = ib;
			}
			else
			{
				float dot1 = vdot( normal1, vsub( vertices[ib1], p1 ) );
				float dot2 = vdot( normal1, vsub( vertices[ib2], p2 ) );
				incidentIndex = dot1 < dot2 ? ib1 : ib2;
			}
		}
	}
	else
	{
		float edgeSeparation = FLT_MAX;
		for ( int i = 0; i < count; ++i )
		{
			float s = vdot( normal1, vsub( vertices[i], p1 ) );
			if ( s < edgeSeparation )
			{
				edgeSeparation = s;
				incidentIndex = i;
			}
		}
		if ( sp.convex1 )
		{
			float s0 = FLT_MAX;
			for ( int i = 0; i < count; ++i )
			{
				float s = vdot( sp.normal0, vsub( vertices[i], p1 ) );
				if ( s < s0 )
					s0 = s;
			}
			if ( s0 > edgeSeparation )
			{
				edgeSeparation = s0;
				incidentIndex = -1;
			}
		}
		if ( sp.convex2 )
		{
			float s2 = FLT_MAX;
			for ( int i = 0; i < count; ++i )
			{
				float s = vdot( sp.normal2, vsub( vertices[i], p2 ) );
				if ( s < s2 )
					s2 = s;
			}
			if ( s2 > edgeSeparation )
			{
				edgeSeparation = s2;
				incidentIndex = -1;
			}
		}
		float polygonSeparation = -FLT_MAX;
		int referenceIndex = -1;
		for ( int i = 0; i < count; ++i )
		{
			fv2 n = normals[i];
			if ( classify_normal( sp, vneg( n ) ) != NORMAL_ADMIT )
				continue;
			fv2 p = vertices[i];
			float s = fmin_s( vdot( n, vsub( p2, p ) ), vdot( n, vsub( p1, p ) ) );
			if ( s > polygonSeparation )
			{
				polygonSeparation = s;
				referenceIndex = i;
			}
		}
		if ( polygonSeparation > edgeSeparation )
		{
			int ia1 = referenceIndex;
			int ia2 = ia1 < count - 1 ? ia1 + 1 : 0;
			fv2 a1 = vertices[ia1];
			fv2 a2 = vertices[ia2];
			fv2 n = normals[ia1];
			float dot1 = vdot( n, vsub( p1, a1 ) );
			float dot2 = vdot( n, vsub( p2, a1 ) );
			if ( dot1 < dot2 )
			{
				if ( vdot( n0, n ) < vdot( normal1, n ) )
					return m;
			}
			else
			{
				if ( vdot( n2, n ) < vdot( normal1, n ) )
					return m;
			}
			m = clip_segments( a1, a2, p1, p2, normals[ia1], radiusB, 0.0f, MAKE_ID( ia1, 1 ), MAKE_ID( ia2, 0 ) );
			finish_clip( m, xfA, xfB, vneg( normals[ia1] ) );
			return m;
		}
		if ( incidentIndex == -1 )
			return m;
	}
	fv2 b1, b2;
	int ib1, ib2;
	if ( incidentNormal != -1 )
	{
		ib1 = incidentNormal;
		ib2 = ib1 < count - 1 ? ib1 + 1 : 0;
		b1 = vertices[ib1];
		b2 = vertices[ib2];
	}
	else
	{
		int i2 = incidentIndex;
		int i1 = i2 > 0 ? i2 - 1 : count - 1;
		float d1 = vdot( normal1, normals[i1] );
		float d2 = vdot( normal1, normals[i2] );
		if ( d1 < d2 )
		{
			ib1 = i1, ib2 = i2;
			b1 = vertices[ib1];
			b2 = vertices[ib2];
		}
		else
		{
			ib1 = i2, ib2 = i2 < count - 1 ? i2 + 1 : 0;
			b1 = vertices[ib1];
			b2 = vertices[ib2];
		}
	}
	m = clip_segments( p1, p2, b1, b2, normal1, 0.0f, radiusB, MAKE_ID( 0, ib2 ), MAKE_ID( 1, ib1 ) );
	finish_clip( m, xfA, xfB, m.normal );
	return m;
}

__device__ __forceinline__ DCache unpack_cache( int2 c )
{
	DCache k;
	k.count = c.x & 0xff;
	for ( int i = 0; i < 3; ++i )
	{
		k.indexA[i] = ( c.x >> ( 8 + 8 * i ) ) & 0xff;
		k.indexB[i] = ( c.y >> ( 8 * i ) ) & 0xff;
	}
	return k;
}

__device__ __forceinline__ int2 pack_cache( const DCache& k )
{
	int2 c;
	c.x = k.count & 0xff;
	c.y = 0;
	for ( int i = 0; i < k.count; ++i )
	{
		c.x |= ( k.indexA[i] & 0xff ) << ( 8 + 8 * i );
		c.y |= ( k.indexB[i] & 0xff ) << ( 8 * i );
	}
	return c;
}

// contact.c:60-148 dispatch; A already carries the registered first type.
// `cache` is the contact's simplex cache, read and written by the chain
// segment manifolds only.
__device__ __forceinline__ DManifold compute_manifold( const DGeom& a, fxf xfA, const DGeom& b, fxf xfB,
													   DCache& cache )
{
	DManifold zero = dm_empty();
	switch ( a.type )
	{
		case ST_CIRCLE:
			if ( b.type == ST_CIRCLE )
				return collide_circles( a.c1, a.radius, xfA, b.c1, b.radius, xfB );
			break;
		case ST_CAPSULE:
			if ( b.type == ST_CIRCLE )
				return collide_capsule_circle( a.c1, a.c2, a.radius, xfA, b.c1, b.radius, xfB );
			if ( b.type == ST_CAPSULE )
				return collide_capsules( a.c1, a.c2, a.radius, xfA, b.c1, b.c2, b.radius, xfB );
			break;
		case ST_POLYGON:
			if ( b.type == ST_CIRCLE )
				return collide_polygon_circle( a.poly, xfA, b.c1, b.radius, xfB );
			if ( b.type == ST_CAPSULE )
			{
				DPoly pb;
				capsule_poly( pb, b.c1, b.c2, b.radius );
				return collide_polygons( a.poly, xfA, pb, xfB );
			}
			if ( b.type == ST_POLYGON )
				return collide_polygons( a.poly, xfA, b.poly, xfB );
			break;
		case ST_SEGMENT:
			if ( b.type == ST_CIRCLE )
				return collide_capsule_circle( a.c1, a.c2, 0.0f, xfA, b.c1, b.radius, xfB );
			if ( b.type == ST_CAPSULE )
				return collide_capsules( a.c1, a.c2, 0.0f, xfA, b.c1, b.c2, b.radius, xfB );
			if ( b.type == ST_POLYGON )
			{
				DPoly pa;
				capsule_poly( pa, a.c1, a.c2, 0.0f );
				return collide_polygons( pa, xfA, b.poly, xfB );
			}
			break;
		case ST_CHAIN:
			if ( b.type == ST_CIRCLE )
				return collide_chain_circle( a, xfA, b.c1, b.radius, xfB );
			if ( b.type == ST_CAPSULE )
			{
				DPoly pb;
				capsule_poly( pb, b.c1, b.c2, b.radius );
				return collide_chain_polygon( a, xfA, pb, vlerp( b.c1, b.c2, 0.5f ), xfB, cache );
			}
			if ( b.type == ST_POLYGON )
				return collide_chain_polygon( a, xfA, b.poly, b.c1, xfB, cache );
			break;
		default:
			break;
	}
	return zero;
}
