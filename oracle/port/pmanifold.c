// Narrowphase manifolds of the restatement. TEST INFRASTRUCTURE (oracle).
// Reference: packages/forge2d/third_party/box2d/src/manifold.c (b2Collide*),
// distance.c:27-97 (b2SegmentDistance), contact.c:126-184 (registry).
#include "port.h"

#define MAKE_ID( A, B ) ( (uint16_t)( ( (uint8_t)( A ) ) << 8 | (uint8_t)( B ) ) )

typedef struct SegDist
{
	v2 closest1, closest2;
	float fraction1, fraction2;
	float distanceSquared;
} SegDist;

// distance.c:27-97
static SegDist segment_distance( v2 p1, v2 q1, v2 p2, v2 q2 )
{
	SegDist r = { 0 };
	v2 d1 = sub( q1, p1 );
	v2 d2 = sub( q2, p2 );
	v2 rr = sub( p1, p2 );
	float dd1 = dot( d1, d1 );
	float dd2 = dot( d2, d2 );
	float rd1 = dot( rr, d1 );
	float rd2 = dot( rr, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	if ( dd1 < epsSqr || dd2 < epsSqr )
	{
		if ( dd1 >= epsSqr )
		{
			r.fraction1 = fclampp( -rd1 / dd1, 0.0f, 1.0f );
			r.fraction2 = 0.0f;
		}
		else if ( dd2 >= epsSqr )
		{
			r.fraction1 = 0.0f;
			r.fraction2 = fclampp( rd2 / dd2, 0.0f, 1.0f );
		}
		else
		{
			r.fraction1 = 0.0f;
			r.fraction2 = 0.0f;
		}
	}
	else
	{
		float d12 = dot( d1, d2 );
		float denom = dd1 * dd2 - d12 * d12;
		float f1 = 0.0f;
		if ( denom != 0.0f )
			f1 = fclampp( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
		float f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2 < 0.0f )
		{
			f2 = 0.0f;
			f1 = fclampp( -rd1 / dd1, 0.0f, 1.0f );
		}
		else if ( f2 > 1.0f )
		{
			f2 = 1.0f;
			f1 = fclampp( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
		}
		r.fraction1 = f1;
		r.fraction2 = f2;
	}
	r.closest1 = mulAdd( p1, r.fraction1, d1 );
	r.closest2 = mulAdd( p2, r.fraction2, d2 );
	r.distanceSquared = distSq( r.closest1, r.closest2 );
	return r;
}

// manifold.c:16-34 (capsule as a 2-gon)
static Polygon make_capsule_poly( v2 p1, v2 p2, float radius )
{
	Polygon s = { 0 };
	s.vertices[0] = p1;
	s.vertices[1] = p2;
	s.centroid = lerp( p1, p2, 0.5f );
	v2 d = sub( p2, p1 );
	v2 axis = normalize( d );
	v2 n = rightPerp( axis );
	s.normals[0] = n;
	s.normals[1] = neg( n );
	s.count = 2;
	s.radius = radius;
	return s;
}

static void finish_point( Manifold* m, xform xfA, xform xfB, v2 contactPointA, float separation, uint16_t id,
						  int pointIsOriginRelative )
{
	ManifoldPoint* mp = m->points + 0;
	mp->anchorA = rotate( xfA.q, contactPointA );
	mp->anchorB = add( mp->anchorA, sub( xfA.p, xfB.p ) );
	mp->point = pointIsOriginRelative ? add( mp->anchorA, xfA.p ) : add( xfA.p, mp->anchorA );
	mp->separation = separation;
	mp->id = id;
	m->pointCount = 1;
}

// manifold.c:40-75
static Manifold collide_circles( v2 centerA, float radiusA, xform xfA, v2 centerB, float radiusB, xform xfB )
{
	Manifold m = { 0 };
	xform xf = invMulXf( xfA, xfB );
	v2 pointA = centerA;
	v2 pointB = xfPoint( xf, centerB );
	float distance;
	v2 normal = lengthAndNormalize( &distance, sub( pointB, pointA ) );
	float separation = distance - radiusA - radiusB;
	if ( separation > P_SPECULATIVE )
		return m;
	v2 cA = mulAdd( pointA, radiusA, normal );
	v2 cB = mulAdd( pointB, -radiusB, normal );
	v2 contactPointA = lerp( cA, cB, 0.5f );
	m.normal = rotate( xfA.q, normal );
	// mp->point = anchorA + xfA.p (operand order as manifold.c:69)
	finish_point( &m, xfA, xfB, contactPointA, separation, 0, 1 );
	return m;
}

// manifold.c:77-139
static Manifold collide_capsule_circle( v2 p1, v2 p2, float radiusA, xform xfA, v2 centerB, float radiusB, xform xfB )
{
	Manifold m = { 0 };
	xform xf = invMulXf( xfA, xfB );
	v2 pB = xfPoint( xf, centerB );
	v2 e = sub( p2, p1 );
	v2 pA;
	float s1 = dot( sub( pB, p1 ), e );
	float s2 = dot( sub( p2, pB ), e );
	if ( s1 < 0.0f )
		pA = p1;
	else if ( s2 < 0.0f )
		pA = p2;
	else
	{
		float s = s1 / dot( e, e );
		pA = mulAdd( p1, s, e );
	}
	float distance;
	v2 normal = lengthAndNormalize( &distance, sub( pB, pA ) );
	float separation = distance - radiusA - radiusB;
	if ( separation > P_SPECULATIVE )
		return m;
	v2 cA = mulAdd( pA, radiusA, normal );
	v2 cB = mulAdd( pB, -radiusB, normal );
	v2 contactPointA = lerp( cA, cB, 0.5f );
	m.normal = rotate( xfA.q, normal );
	finish_point( &m, xfA, xfB, contactPointA, separation, 0, 0 );
	return m;
}

// manifold.c:141-259
static Manifold collide_polygon_circle( const Polygon* polyA, xform xfA, v2 centerB, float radiusB, xform xfB )
{
	Manifold m = { 0 };
	xform xf = invMulXf( xfA, xfB );
	v2 center = xfPoint( xf, centerB );
	float radiusA = polyA->radius;
	float radius = radiusA + radiusB;
	int normalIndex = 0;
	float separation = -FLT_MAX;
	int vc = polyA->count;
	const v2* vs = polyA->vertices;
	const v2* ns = polyA->normals;
	for ( int i = 0; i < vc; ++i )
	{
		float s = dot( ns[i], sub( center, vs[i] ) );
		if ( s > separation )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation > radius + P_SPECULATIVE )
		return m;
	int i1 = normalIndex;
	int i2 = i1 + 1 < vc ? i1 + 1 : 0;
	v2 v1 = vs[i1];
	v2 v2p = vs[i2];
	float u1 = dot( sub( center, v1 ), sub( v2p, v1 ) );
	float u2 = dot( sub( center, v2p ), sub( v1, v2p ) );
	if ( u1 < 0.0f && separation > FLT_EPSILON )
	{
		v2 normal = normalize( sub( center, v1 ) );
		separation = dot( sub( center, v1 ), normal );
		if ( separation > radius + P_SPECULATIVE )
			return m;
		v2 cA = mulAdd( v1, radiusA, normal );
		v2 cB = mulSub( center, radiusB, normal );
		v2 cp = lerp( cA, cB, 0.5f );
		m.normal = rotate( xfA.q, normal );
		finish_point( &m, xfA, xfB, cp, dot( sub( cB, cA ), normal ), 0, 0 );
	}
	else if ( u2 < 0.0f && separation > FLT_EPSILON )
	{
		v2 normal = normalize( sub( center, v2p ) );
		separation = dot( sub( center, v2p ), normal );
		if ( separation > radius + P_SPECULATIVE )
			return m;
		v2 cA = mulAdd( v2p, radiusA, normal );
		v2 cB = mulSub( center, radiusB, normal );
		v2 cp = lerp( cA, cB, 0.5f );
		m.normal = rotate( xfA.q, normal );
		finish_point( &m, xfA, xfB, cp, dot( sub( cB, cA ), normal ), 0, 0 );
	}
	else
	{
		v2 normal = ns[normalIndex];
		m.normal = rotate( xfA.q, normal );
		v2 cA = mulAdd( center, radiusA - dot( sub( center, v1 ), normal ), normal );
		v2 cB = mulSub( center, radiusB, normal );
		v2 cp = lerp( cA, cB, 0.5f );
		finish_point( &m, xfA, xfB, cp, separation - radius, 0, 0 );
	}
	return m;
}

// manifold.c:261-530 (segment-segment closest points with clipping)
static Manifold collide_capsules( v2 a1, v2 a2, float radiusA, xform xfA, v2 b1, v2 b2, float radiusB, xform xfB )
{
	v2 origin = a1;
	xform sfA = { add( xfA.p, rotate( xfA.q, origin ) ), xfA.q };
	xform xf = invMulXf( sfA, xfB );
	v2 p1 = V( 0.0f, 0.0f );
	v2 q1 = sub( a2, origin );
	v2 p2 = xfPoint( xf, b1 );
	v2 q2 = xfPoint( xf, b2 );
	v2 d1 = sub( q1, p1 );
	v2 d2 = sub( q2, p2 );
	float dd1 = dot( d1, d1 );
	float dd2 = dot( d2, d2 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	v2 r = sub( p1, p2 );
	float rd1 = dot( r, d1 );
	float rd2 = dot( r, d2 );
	float d12 = dot( d1, d2 );
	float denom = dd1 * dd2 - d12 * d12;
	float f1 = 0.0f;
	if ( denom != 0.0f )
		f1 = fclampp( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
	float f2 = ( d12 * f1 + rd2 ) / dd2;
	if ( f2 < 0.0f )
	{
		f2 = 0.0f;
		f1 = fclampp( -rd1 / dd1, 0.0f, 1.0f );
	}
	else if ( f2 > 1.0f )
	{
		f2 = 1.0f;
		f1 = fclampp( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
	}
	v2 closest1 = mulAdd( p1, f1, d1 );
	v2 closest2 = mulAdd( p2, f2, d2 );
	float distanceSquared = distSq( closest1, closest2 );
	Manifold m = { 0 };
	float radius = radiusA + radiusB;
	float maxDistance = radius + P_SPECULATIVE;
	if ( distanceSquared > maxDistance * maxDistance )
		return m;
	float distance = sqrtf( distanceSquared );
	float length1, length2;
	v2 u1 = lengthAndNormalize( &length1, d1 );
	v2 u2 = lengthAndNormalize( &length2, d2 );
	float fp2 = dot( sub( p2, p1 ), u1 );
	float fq2 = dot( sub( q2, p1 ), u1 );
	bool outsideA = ( fp2 <= 0.0f && fq2 <= 0.0f ) || ( fp2 >= length1 && fq2 >= length1 );
	float fp1 = dot( sub( p1, p2 ), u2 );
	float fq1 = dot( sub( q1, p2 ), u2 );
	bool outsideB = ( fp1 <= 0.0f && fq1 <= 0.0f ) || ( fp1 >= length2 && fq1 >= length2 );
	if ( outsideA == false && outsideB == false )
	{
		v2 normalA;
		float separationA;
		{
			normalA = leftPerp( u1 );
			float ss1 = dot( sub( p2, p1 ), normalA );
			float ss2 = dot( sub( q2, p1 ), normalA );
			float s1p = ss1 < ss2 ? ss1 : ss2;
			float s1n = -ss1 < -ss2 ? -ss1 : -ss2;
			if ( s1p > s1n )
				separationA = s1p;
			else
			{
				separationA = s1n;
				normalA = neg( normalA );
			}
		}
		v2 normalB;
		float separationB;
		{
			normalB = leftPerp( u2 );
			float ss1 = dot( sub( p1, p2 ), normalB );
			float ss2 = dot( sub( q1, p2 ), normalB );
			float s1p = ss1 < ss2 ? ss1 : ss2;
			float s1n = -ss1 < -ss2 ? -ss1 : -ss2;
			if ( s1p > s1n )
				separationB = s1p;
			else
			{
				separationB = s1n;
				normalB = neg( normalB );
			}
		}
		if ( separationA + 0.1f * P_LINEAR_SLOP >= separationB )
		{
			m.normal = normalA;
			v2 cp = p2;
			v2 cq = q2;
			if ( fp2 < 0.0f && fq2 > 0.0f )
				cp = lerp( p2, q2, ( 0.0f - fp2 ) / ( fq2 - fp2 ) );
			else if ( fq2 < 0.0f && fp2 > 0.0f )
				cq = lerp( q2, p2, ( 0.0f - fq2 ) / ( fp2 - fq2 ) );
			if ( fp2 > length1 && fq2 < length1 )
				cp = lerp( p2, q2, ( fp2 - length1 ) / ( fp2 - fq2 ) );
			else if ( fq2 > length1 && fp2 < length1 )
				cq = lerp( q2, p2, ( fq2 - length1 ) / ( fq2 - fp2 ) );
			float sp = dot( sub( cp, p1 ), normalA );
			float sq = dot( sub( cq, p1 ), normalA );
			if ( sp <= distance + P_LINEAR_SLOP || sq <= distance + P_LINEAR_SLOP )
			{
				ManifoldPoint* mp = m.points + 0;
				mp->anchorA = mulAdd( cp, 0.5f * ( radiusA - radiusB - sp ), normalA );
				mp->separation = sp - radius;
				mp->id = MAKE_ID( 0, 0 );
				mp = m.points + 1;
				mp->anchorA = mulAdd( cq, 0.5f * ( radiusA - radiusB - sq ), normalA );
				mp->separation = sq - radius;
				mp->id = MAKE_ID( 0, 1 );
				m.pointCount = 2;
			}
		}
		else
		{
			m.normal = neg( normalB );
			v2 cp = p1;
			v2 cq = q1;
			if ( fp1 < 0.0f && fq1 > 0.0f )
				cp = lerp( p1, q1, ( 0.0f - fp1 ) / ( fq1 - fp1 ) );
			else if ( fq1 < 0.0f && fp1 > 0.0f )
				cq = lerp( q1, p1, ( 0.0f - fq1 ) / ( fp1 - fq1 ) );
			if ( fp1 > length2 && fq1 < length2 )
				cp = lerp( p1, q1, ( fp1 - length2 ) / ( fp1 - fq1 ) );
			else if ( fq1 > length2 && fp1 < length2 )
				cq = lerp( q1, p1, ( fq1 - length2 ) / ( fq1 - fp1 ) );
			float sp = dot( sub( cp, p2 ), normalB );
			float sq = dot( sub( cq, p2 ), normalB );
			if ( sp <= distance + P_LINEAR_SLOP || sq <= distance + P_LINEAR_SLOP )
			{
				ManifoldPoint* mp = m.points + 0;
				mp->anchorA = mulAdd( cp, 0.5f * ( radiusB - radiusA - sp ), normalB );
				mp->separation = sp - radius;
				mp->id = MAKE_ID( 0, 0 );
				mp = m.points + 1;
				mp->anchorA = mulAdd( cq, 0.5f * ( radiusB - radiusA - sq ), normalB );
				mp->separation = sq - radius;
				mp->id = MAKE_ID( 1, 0 );
				m.pointCount = 2;
			}
		}
	}
	if ( m.pointCount == 0 )
	{
		v2 normal = sub( closest2, closest1 );
		if ( dot( normal, normal ) > epsSqr )
			normal = normalize( normal );
		else
			normal = leftPerp( u1 );
		v2 c1 = mulAdd( closest1, radiusA, normal );
		v2 c2 = mulAdd( closest2, -radiusB, normal );
		int i1 = f1 == 0.0f ? 0 : 1;
		int i2 = f2 == 0.0f ? 0 : 1;
		m.normal = normal;
		m.points[0].anchorA = lerp( c1, c2, 0.5f );
		m.points[0].separation = sqrtf( distanceSquared ) - radius;
		m.points[0].id = MAKE_ID( i1, i2 );
		m.pointCount = 1;
	}
	m.normal = rotate( xfA.q, m.normal );
	for ( int i = 0; i < m.pointCount; ++i )
	{
		ManifoldPoint* mp = m.points + i;
		mp->anchorA = rotate( xfA.q, add( mp->anchorA, origin ) );
		mp->anchorB = add( mp->anchorA, sub( xfA.p, xfB.p ) );
		mp->point = add( xfA.p, mp->anchorA );
	}
	return m;
}

// manifold.c:545-678 (b2ClipPolygons)
static Manifold clip_polygons( const Polygon* polyA, const Polygon* polyB, int edgeA, int edgeB, bool flip )
{
	Manifold m = { 0 };
	const Polygon* poly1;
	int i11, i12;
	const Polygon* poly2;
	int i21, i22;
	if ( flip )
	{
		poly1 = polyB;
		poly2 = polyA;
		i11 = edgeB;
		i12 = edgeB + 1 < polyB->count ? edgeB + 1 : 0;
		i21 = edgeA;
		i22 = edgeA + 1 < polyA->count ? edgeA + 1 : 0;
	}
	else
	{
		poly1 = polyA;
		poly2 = polyB;
		i11 = edgeA;
		i12 = edgeA + 1 < polyA->count ? edgeA + 1 : 0;
		i21 = edgeB;
		i22 = edgeB + 1 < polyB->count ? edgeB + 1 : 0;
	}
	v2 normal = poly1->normals[i11];
	v2 v11 = poly1->vertices[i11];
	v2 v12 = poly1->vertices[i12];
	v2 v21 = poly2->vertices[i21];
	v2 v22 = poly2->vertices[i22];
	v2 tangent = crossSV( 1.0f, normal );
	float lower1 = 0.0f;
	float upper1 = dot( sub( v12, v11 ), tangent );
	float upper2 = dot( sub( v21, v11 ), tangent );
	float lower2 = dot( sub( v22, v11 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 )
		return m;
	v2 vLower;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON )
		vLower = lerp( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = v22;
	v2 vUpper;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON )
		vUpper = lerp( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = v21;
	float separationLower = dot( sub( vLower, v11 ), normal );
	float separationUpper = dot( sub( vUpper, v11 ), normal );
	float r1 = poly1->radius;
	float r2 = poly2->radius;
	vLower = mulAdd( vLower, 0.5f * ( r1 - r2 - separationLower ), normal );
	vUpper = mulAdd( vUpper, 0.5f * ( r1 - r2 - separationUpper ), normal );
	float radius = r1 + r2;
	if ( flip == false )
	{
		m.normal = normal;
		m.points[0].anchorA = vLower;
		m.points[0].separation = separationLower - radius;
		m.points[0].id = MAKE_ID( i11, i22 );
		m.points[1].anchorA = vUpper;
		m.points[1].separation = separationUpper - radius;
		m.points[1].id = MAKE_ID( i12, i21 );
		m.pointCount = 2;
	}
	else
	{
		m.normal = neg( normal );
		m.points[0].anchorA = vUpper;
		m.points[0].separation = separationUpper - radius;
		m.points[0].id = MAKE_ID( i21, i12 );
		m.points[1].anchorA = vLower;
		m.points[1].separation = separationLower - radius;
		m.points[1].id = MAKE_ID( i22, i11 );
		m.pointCount = 2;
	}
	return m;
}

// manifold.c:680-718 (b2FindMaxSeparation)
static float find_max_separation( int* edgeIndex, const Polygon* poly1, const Polygon* poly2 )
{
	int count1 = poly1->count;
	int count2 = poly2->count;
	int bestIndex = 0;
	float maxSeparation = -FLT_MAX;
	for ( int i = 0; i < count1; ++i )
	{
		v2 n = poly1->normals[i];
		v2 v1 = poly1->vertices[i];
		float si = FLT_MAX;
		for ( int j = 0; j < count2; ++j )
		{
			float sij = dot( n, sub( poly2->vertices[j], v1 ) );
			if ( sij < si )
				si = sij;
		}
		if ( si > maxSeparation )
		{
			maxSeparation = si;
			bestIndex = i;
		}
	}
	*edgeIndex = bestIndex;
	return maxSeparation;
}

static void vertex_vertex( Manifold* m, v2 va, v2 vb, float ra, float rb, float distance, float radius, uint16_t id )
{
	v2 normal = sub( vb, va );
	float invDistance = 1.0f / distance;
	normal.x *= invDistance;
	normal.y *= invDistance;
	v2 c1 = mulAdd( va, ra, normal );
	v2 c2 = mulAdd( vb, -rb, normal );
	m->normal = normal;
	m->points[0].anchorA = lerp( c1, c2, 0.5f );
	m->points[0].separation = distance - radius;
	m->points[0].id = id;
	m->pointCount = 1;
}

// manifold.c:736-1075 (b2CollidePolygons, the "#if 1" branch)
static Manifold collide_polygons( const Polygon* polygonA, xform xfA, const Polygon* polygonB, xform xfB )
{
	v2 origin = polygonA->vertices[0];
	const float linearSlop = P_LINEAR_SLOP;
	const float speculativeDistance = P_SPECULATIVE;
	xform sfA = { add( xfA.p, rotate( xfA.q, origin ) ), xfA.q };
	xform xf = invMulXf( sfA, xfB );
	Polygon la;
	la.count = polygonA->count;
	la.radius = polygonA->radius;
	la.vertices[0] = V( 0.0f, 0.0f );
	la.normals[0] = polygonA->normals[0];
	for ( int i = 1; i < la.count; ++i )
	{
		la.vertices[i] = sub( polygonA->vertices[i], origin );
		la.normals[i] = polygonA->normals[i];
	}
	Polygon lb;
	lb.count = polygonB->count;
	lb.radius = polygonB->radius;
	for ( int i = 0; i < lb.count; ++i )
	{
		lb.vertices[i] = xfPoint( xf, polygonB->vertices[i] );
		lb.normals[i] = rotate( xf.q, polygonB->normals[i] );
	}
	int edgeA = 0;
	float separationA = find_max_separation( &edgeA, &la, &lb );
	int edgeB = 0;
	float separationB = find_max_separation( &edgeB, &lb, &la );
	float radius = la.radius + lb.radius;
	Manifold m = { 0 };
	if ( separationA > speculativeDistance + radius || separationB > speculativeDistance + radius )
		return m;
	bool flip;
	if ( separationA >= separationB )
	{
		flip = false;
		v2 searchDirection = la.normals[edgeA];
		edgeB = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < lb.count; ++i )
		{
			float d = dot( searchDirection, lb.normals[i] );
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
		v2 searchDirection = lb.normals[edgeB];
		edgeA = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < la.count; ++i )
		{
			float d = dot( searchDirection, la.normals[i] );
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}
	if ( separationA > 0.1f * linearSlop || separationB > 0.1f * linearSlop )
	{
		int i11 = edgeA;
		int i12 = edgeA + 1 < la.count ? edgeA + 1 : 0;
		int i21 = edgeB;
		int i22 = edgeB + 1 < lb.count ? edgeB + 1 : 0;
		v2 v11 = la.vertices[i11];
		v2 v12 = la.vertices[i12];
		v2 v21 = lb.vertices[i21];
		v2 v22 = lb.vertices[i22];
		SegDist result = segment_distance( v11, v12, v21, v22 );
		float distance = sqrtf( result.distanceSquared );
		float separation = distance - radius;
		if ( distance - radius > speculativeDistance )
			return m;
		m = clip_polygons( &la, &lb, edgeA, edgeB, flip );
		float minSeparation = FLT_MAX;
		for ( int i = 0; i < m.pointCount; ++i )
			minSeparation = fminp( minSeparation, m.points[i].separation );
		if ( separation + 0.1f * linearSlop < minSeparation )
		{
			if ( result.fraction1 == 0.0f && result.fraction2 == 0.0f )
				vertex_vertex( &m, v11, v21, la.radius, lb.radius, distance, radius, MAKE_ID( i11, i21 ) );
			else if ( result.fraction1 == 0.0f && result.fraction2 == 1.0f )
				vertex_vertex( &m, v11, v22, la.radius, lb.radius, distance, radius, MAKE_ID( i11, i22 ) );
			else if ( result.fraction1 == 1.0f && result.fraction2 == 0.0f )
				vertex_vertex( &m, v12, v21, la.radius, lb.radius, distance, radius, MAKE_ID( i12, i21 ) );
			else if ( result.fraction1 == 1.0f && result.fraction2 == 1.0f )
				vertex_vertex( &m, v12, v22, la.radius, lb.radius, distance, radius, MAKE_ID( i12, i22 ) );
		}
	}
	else
	{
		m = clip_polygons( &la, &lb, edgeA, edgeB, flip );
	}
	if ( m.pointCount > 0 )
	{
		m.normal = rotate( xfA.q, m.normal );
		for ( int i = 0; i < m.pointCount; ++i )
		{
			ManifoldPoint* mp = m.points + i;
			mp->anchorA = rotate( xfA.q, add( mp->anchorA, origin ) );
			mp->anchorB = add( mp->anchorA, sub( xfA.p, xfB.p ) );
			mp->point = add( xfA.p, mp->anchorA );
		}
	}
	return m;
}

// manifold.c:1089-1168: one-sided, with the ghost vertices' Voronoi regions
static Manifold collide_chain_circle( const Geometry* segA, xform xfA, v2 centerB, float radius, xform xfB )
{
	Manifold m = { 0 };
	xform xf = invMulXf( xfA, xfB );
	v2 pB = xfPoint( xf, centerB );
	v2 p1 = segA->c1;
	v2 p2 = segA->c2;
	v2 e = sub( p2, p1 );
	float offset = dot( rightPerp( e ), sub( pB, p1 ) );
	if ( offset < 0.0f )
		return m;
	float u = dot( e, sub( p2, pB ) );
	float v = dot( e, sub( pB, p1 ) );
	v2 pA;
	if ( v <= 0.0f )
	{
		v2 prevEdge = sub( p1, segA->g1 );
		float uPrev = dot( prevEdge, sub( pB, p1 ) );
		if ( uPrev <= 0.0f )
			return m;
		pA = p1;
	}
	else if ( u <= 0.0f )
	{
		v2 nextEdge = sub( segA->g2, p2 );
		float vNext = dot( nextEdge, sub( pB, p2 ) );
		if ( vNext > 0.0f )
			return m;
		pA = p2;
	}
	else
	{
		float ee = dot( e, e );
		pA = V( u * p1.x + v * p2.x, u * p1.y + v * p2.y );
		pA = ee > 0.0f ? mulSV( 1.0f / ee, pA ) : p1;
	}
	float distance;
	v2 normal = lengthAndNormalize( &distance, sub( pB, pA ) );
	float separation = distance - radius;
	if ( separation > P_SPECULATIVE )
		return m;
	v2 cA = pA;
	v2 cB = mulAdd( pB, -radius, normal );
	v2 contactPointA = lerp( cA, cB, 0.5f );
	m.normal = rotate( xfA.q, normal );
	finish_point( &m, xfA, xfB, contactPointA, separation, 0, 0 );
	return m;
}

// manifold.c:1177-1254 b2ClipSegments (points in the frame of A, unrotated)
static Manifold clip_segments( v2 a1, v2 a2, v2 b1, v2 b2, v2 normal, float ra, float rb, uint16_t id1,
							   uint16_t id2 )
{
	Manifold m = { 0 };
	v2 tangent = leftPerp( normal );
	float lower1 = 0.0f;
	float upper1 = dot( sub( a2, a1 ), tangent );
	float upper2 = dot( sub( b1, a1 ), tangent );
	float lower2 = dot( sub( b2, a1 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 )
		return m;
	v2 vLower;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON )
		vLower = lerp( b2, b1, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = b2;
	v2 vUpper;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON )
		vUpper = lerp( b2, b1, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = b1;
	float separationLower = dot( sub( vLower, a1 ), normal );
	float separationUpper = dot( sub( vUpper, a1 ), normal );
	vLower = mulAdd( vLower, 0.5f * ( ra - rb - separationLower ), normal );
	vUpper = mulAdd( vUpper, 0.5f * ( ra - rb - separationUpper ), normal );
	float radius = ra + rb;
	m.normal = normal;
	m.points[0].anchorA = vLower;
	m.points[0].separation = separationLower - radius;
	m.points[0].id = id1;
	m.points[1].anchorA = vUpper;
	m.points[1].separation = separationUpper - radius;
	m.points[1].id = id2;
	m.pointCount = 2;
	return m;
}

enum
{
	NORMAL_SKIP = 0,
	NORMAL_ADMIT = 1,
	NORMAL_SNAP = 2,
};

typedef struct ChainParams
{
	v2 edge1, normal0, normal2;
	int convex1, convex2;
} ChainParams;

// manifold.c:1270-1316 b2ClassifyNormal (Gauss map of the chain vertex)
static int classify_normal( const ChainParams* p, v2 normal )
{
	const float sinTol = 0.01f;
	if ( dot( normal, p->edge1 ) <= 0.0f )
	{
		if ( p->convex1 )
			return cross( normal, p->normal0 ) > sinTol ? NORMAL_SKIP : NORMAL_ADMIT;
		return NORMAL_SNAP;
	}
	if ( p->convex2 )
		return cross( p->normal2, normal ) > sinTol ? NORMAL_SKIP : NORMAL_ADMIT;
	return NORMAL_SNAP;
}

// rotates a clipped two-point manifold from the segment frame to the world
static void finish_clip( Manifold* m, xform xfA, xform xfB, v2 normalLocal )
{
	if ( m->pointCount != 2 )
		return;
	m->normal = rotate( xfA.q, normalLocal );
	m->points[0].anchorA = rotate( xfA.q, m->points[0].anchorA );
	m->points[1].anchorA = rotate( xfA.q, m->points[1].anchorA );
	v2 pAB = sub( xfA.p, xfB.p );
	m->points[0].anchorB = add( m->points[0].anchorA, pAB );
	m->points[1].anchorB = add( m->points[1].anchorA, pAB );
	m->points[0].point = add( xfA.p, m->points[0].anchorA );
	m->points[1].point = add( xfA.p, m->points[1].anchorA );
}

// manifold.c:1318-1726 b2CollideChainSegmentAndPolygon: GJK (warm-started
// from the contact's simplex cache) picks vertex-vertex, vertex-edge or the
// SAT over the segment normal, its convex neighbours and the admitted
// polygon normals; ghost collisions are skipped or snapped by the Gauss map
static Manifold collide_chain_polygon( const Geometry* segA, xform xfA, const Polygon* polygonB, xform xfB,
									   SimplexCache* cache )
{
	Manifold m = { 0 };
	xform xf = invMulXf( xfA, xfB );
	v2 centroidB = xfPoint( xf, polygonB->centroid );
	float radiusB = polygonB->radius;
	v2 p1 = segA->c1;
	v2 p2 = segA->c2;
	v2 edge1 = normalize( sub( p2, p1 ) );
	ChainParams sp = { 0 };
	sp.edge1 = edge1;
	const float convexTol = 0.01f;
	v2 edge0 = normalize( sub( p1, segA->g1 ) );
	sp.normal0 = rightPerp( edge0 );
	sp.convex1 = cross( edge0, edge1 ) >= convexTol;
	v2 edge2 = normalize( sub( segA->g2, p2 ) );
	sp.normal2 = rightPerp( edge2 );
	sp.convex2 = cross( edge1, edge2 ) >= convexTol;
	v2 normal1 = rightPerp( edge1 );
	int behind1 = dot( normal1, sub( centroidB, p1 ) ) < 0.0f;
	int behind0 = 1, behind2 = 1;
	if ( sp.convex1 )
		behind0 = dot( sp.normal0, sub( centroidB, p1 ) ) < 0.0f;
	if ( sp.convex2 )
		behind2 = dot( sp.normal2, sub( centroidB, p2 ) ) < 0.0f;
	if ( behind1 && behind0 && behind2 )
		return m;
	int count = polygonB->count;
	v2 vertices[P_MAX_POLY];
	v2 normals[P_MAX_POLY];
	for ( int i = 0; i < count; ++i )
	{
		vertices[i] = xfPoint( xf, polygonB->vertices[i] );
		normals[i] = rotate( xf.q, polygonB->normals[i] );
	}
	ShapeProxy proxyA = p_make_proxy( &segA->c1, 2, 0.0f );
	ShapeProxy proxyB = p_make_proxy( vertices, count, 0.0f );
	xform identity = { { 0.0f, 0.0f }, { 1.0f, 0.0f } };
	v2 pointA = V( 0.0f, 0.0f ), pointB = V( 0.0f, 0.0f );
	float distance = p_shape_distance( &proxyA, &proxyB, identity, identity, cache, &pointA, &pointB, 0 );
	if ( distance > radiusB + P_SPECULATIVE )
		return m;
	v2 n0 = sp.convex1 ? sp.normal0 : normal1;
	v2 n2 = sp.convex2 ? sp.normal2 : normal1;
	int incidentIndex = -1;
	int incidentNormal = -1;
	if ( behind1 == 0 && distance > 0.1f * P_LINEAR_SLOP )
	{
		if ( cache->count == 1 )
		{
			v2 pA = pointA;
			v2 pB = pointB;
			v2 normal = normalize( sub( pB, pA ) );
			int type = classify_normal( &sp, normal );
			if ( type == NORMAL_SKIP )
				return m;
			if ( type == NORMAL_ADMIT )
			{
				m.normal = rotate( xfA.q, normal );
				ManifoldPoint* cp = m.points + 0;
				cp->anchorA = rotate( xfA.q, pA );
				cp->anchorB = add( cp->anchorA, sub( xfA.p, xfB.p ) );
				cp->point = add( xfA.p, cp->anchorA );
				cp->separation = distance - radiusB;
				cp->id = MAKE_ID( cache->indexA[0], cache->indexB[0] );
				m.pointCount = 1;
				return m;
			}
			incidentIndex = cache->indexB[0];
		}
		else
		{
			int ia1 = cache->indexA[0];
			int ia2 = cache->indexA[1];
			int ib1 = cache->indexB[0];
			int ib2 = cache->indexB[1];
			if ( ia1 == ia2 )
			{
				v2 normalB = sub( pointA, pointB );
				float dot1 = dot( normalB, normals[ib1] );
				float dot2 = dot( normalB, normals[ib2] );
				int ib = dot1 > dot2 ? ib1 : ib2;
				normalB = normals[ib];
				int type = classify_normal( &sp, neg( normalB ) );
				if ( type == NORMAL_SKIP )
					return m;
				if ( type == NORMAL_ADMIT )
				{
					ib1 = ib;
					ib2 = ib < count - 1 ? ib + 1 : 0;
					v2 b1 = vertices[ib1];
					v2 b2 = vertices[ib2];
					dot1 = dot( normalB, sub( p1, b1 ) );
					dot2 = dot( normalB, sub( p2, b1 ) );
					if ( dot1 < dot2 )
					{
						if ( dot( n0, normalB ) < dot( normal1, normalB ) )
							return m;
					}
					else
					{
						if ( dot( n2, normalB ) < dot( normal1, normalB ) )
							return m;
					}
					m = clip_segments( b1, b2, p1, p2, normalB, radiusB, 0.0f, MAKE_ID( ib1, 1 ), MAKE_ID( ib2, 0 ) );
					finish_clip( &m, xfA, xfB, neg( normalB ) );
					return m;
				}
				incidentNormal = ib;
			}
			else
			{
				float dot1 = dot( normal1, sub( vertices[ib1], p1 ) );
				float dot2 = dot( normal1, sub( vertices[ib2], p2 ) );
				incidentIndex = dot1 < dot2 ? ib1 : ib2;
			}
		}
	}
	else
	{
		float edgeSeparation = FLT_MAX;
		for ( int i = 0; i < count; ++i )
		{
			float s = dot( normal1, sub( vertices[i], p1 ) );
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
				float s = dot( sp.normal0, sub( vertices[i], p1 ) );
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
				float s = dot( sp.normal2, sub( vertices[i], p2 ) );
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
			v2 n = normals[i];
			if ( classify_normal( &sp, neg( n ) ) != NORMAL_ADMIT )
				continue;
			v2 p = vertices[i];
			float s = fminp( dot( n, sub( p2, p ) ), dot( n, sub( p1, p ) ) );
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
			v2 a1 = vertices[ia1];
			v2 a2 = vertices[ia2];
			v2 n = normals[ia1];
			float dot1 = dot( n, sub( p1, a1 ) );
			float dot2 = dot( n, sub( p2, a1 ) );
			if ( dot1 < dot2 )
			{
				if ( dot( n0, n ) < dot( normal1, n ) )
					return m;
			}
			else
			{
				if ( dot( n2, n ) < dot( normal1, n ) )
					return m;
			}
			m = clip_segments( a1, a2, p1, p2, normals[ia1], radiusB, 0.0f, MAKE_ID( ia1, 1 ), MAKE_ID( ia2, 0 ) );
			finish_clip( &m, xfA, xfB, neg( normals[ia1] ) );
			return m;
		}
		if ( incidentIndex == -1 )
			return m;
	}
	v2 b1, b2;
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
		float d1 = dot( normal1, normals[i1] );
		float d2 = dot( normal1, normals[i2] );
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
	finish_clip( &m, xfA, xfB, m.normal );
	return m;
}

// contact.c:126-152: the manifold function registry. Returns nonzero when a
// function exists for (typeA, typeB); *primary is 0 when the pair must be
// flipped so that A has the registered first type.
int p_manifold_registered( int typeA, int typeB, int* primary )
{
	// registered (first, second): circle-circle, capsule-circle, capsule-capsule,
	// polygon-circle, polygon-capsule, polygon-polygon, segment-circle,
	// segment-capsule, segment-polygon, chain-circle, chain-capsule,
	// chain-polygon
	static const int reg[5][5] = {
		//            circle capsule segment polygon chain
		/* circle  */ { 1, 0, 0, 0, 0 },
		/* capsule */ { 1, 1, 0, 0, 0 },
		/* segment */ { 1, 1, 0, 1, 0 },
		/* polygon */ { 1, 1, 0, 1, 0 },
		/* chain   */ { 1, 1, 0, 1, 0 },
	};
	if ( reg[typeA][typeB] )
	{
		*primary = 1;
		return 1;
	}
	if ( reg[typeB][typeA] )
	{
		*primary = 0;
		return 1;
	}
	*primary = 1;
	return 0;
}

// contact.c:60-124 dispatch (A already has the primary type)
Manifold p_collide( const Geometry* a, xform xfA, const Geometry* b, xform xfB, SimplexCache* cache )
{
	Manifold zero = { 0 };
	switch ( a->type )
	{
		case SHAPE_CIRCLE:
			if ( b->type == SHAPE_CIRCLE )
				return collide_circles( a->c1, a->radius, xfA, b->c1, b->radius, xfB );
			break;
		case SHAPE_CAPSULE:
			if ( b->type == SHAPE_CIRCLE )
				return collide_capsule_circle( a->c1, a->c2, a->radius, xfA, b->c1, b->radius, xfB );
			if ( b->type == SHAPE_CAPSULE )
				return collide_capsules( a->c1, a->c2, a->radius, xfA, b->c1, b->c2, b->radius, xfB );
			break;
		case SHAPE_POLYGON:
			if ( b->type == SHAPE_CIRCLE )
				return collide_polygon_circle( &a->poly, xfA, b->c1, b->radius, xfB );
			if ( b->type == SHAPE_CAPSULE )
			{
				Polygon pb = make_capsule_poly( b->c1, b->c2, b->radius );
				return collide_polygons( &a->poly, xfA, &pb, xfB );
			}
			if ( b->type == SHAPE_POLYGON )
				return collide_polygons( &a->poly, xfA, &b->poly, xfB );
			break;
		case SHAPE_SEGMENT:
			if ( b->type == SHAPE_CIRCLE )
				return collide_capsule_circle( a->c1, a->c2, 0.0f, xfA, b->c1, b->radius, xfB );
			if ( b->type == SHAPE_CAPSULE )
				return collide_capsules( a->c1, a->c2, 0.0f, xfA, b->c1, b->c2, b->radius, xfB );
			if ( b->type == SHAPE_POLYGON )
			{
				Polygon pa = make_capsule_poly( a->c1, a->c2, 0.0f );
				return collide_polygons( &pa, xfA, &b->poly, xfB );
			}
			break;
		case SHAPE_CHAIN_SEGMENT:
			if ( b->type == SHAPE_CIRCLE )
				return collide_chain_circle( a, xfA, b->c1, b->radius, xfB );
			if ( b->type == SHAPE_CAPSULE )
			{
				Polygon pb = make_capsule_poly( b->c1, b->c2, b->radius );
				return collide_chain_polygon( a, xfA, &pb, xfB, cache );
			}
			if ( b->type == SHAPE_POLYGON )
				return collide_chain_polygon( a, xfA, &b->poly, xfB, cache );
			break;
		default:
			break;
	}
	return zero;
}
