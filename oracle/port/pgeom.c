// Geometry of the restatement: deterministic trig, convex hull, polygon
// construction, mass properties, AABBs and extents. TEST INFRASTRUCTURE
// (oracle). Reference: packages/forge2d/third_party/box2d/src/
// math_functions.c, hull.c, geometry.c, shape.c.
#include "port.h"

// math_functions.c:61-102: minimax polynomial atan2 (11-bit accurate)
float p_atan2( float y, float x )
{
	if ( x == 0.0f && y == 0.0f )
		return 0.0f;
	float ax = fabsp( x );
	float ay = fabsp( y );
	float mx = fmaxp( ay, ax );
	float mn = fminp( ay, ax );
	float a = mn / mx;
	float s = a * a;
	float c = s * a;
	float q = s * s;
	float r = 0.024840285f * q + 0.18681418f;
	float t = -0.094097948f * q - 0.33213072f;
	r = r * s + t;
	r = r * c + a;
	if ( ay > ax )
		r = 1.57079637f - r;
	if ( x < 0 )
		r = 3.14159274f - r;
	if ( y < 0 )
		r = -r;
	return r;
}

// math_functions.c:108-151: Bhaskara-I approximation, renormalised
void p_cossin( float radians, float* cosOut, float* sinOut )
{
	float x = unwindAngle( radians );
	float pi2 = P_PI * P_PI;
	float c;
	if ( x < -0.5f * P_PI )
	{
		float y = x + P_PI;
		float y2 = y * y;
		c = -( pi2 - 4.0f * y2 ) / ( pi2 + y2 );
	}
	else if ( x > 0.5f * P_PI )
	{
		float y = x - P_PI;
		float y2 = y * y;
		c = -( pi2 - 4.0f * y2 ) / ( pi2 + y2 );
	}
	else
	{
		float y2 = x * x;
		c = ( pi2 - 4.0f * y2 ) / ( pi2 + y2 );
	}
	float s;
	if ( x < 0.0f )
	{
		float y = x + P_PI;
		s = -16.0f * y * ( P_PI - y ) / ( 5.0f * pi2 - 4.0f * y * ( P_PI - y ) );
	}
	else
	{
		s = 16.0f * x * ( P_PI - x ) / ( 5.0f * pi2 - 4.0f * x * ( P_PI - x ) );
	}
	float mag = sqrtf( s * s + c * c );
	float invMag = mag > 0.0f ? 1.0f / mag : 0.0f;
	*cosOut = c * invMag;
	*sinOut = s * invMag;
}

// hull.c:12-71: quickhull recursion on the points right of p1->p2
static int hull_recurse( v2 p1, v2 p2, const v2* ps, int count, v2* out )
{
	if ( count == 0 )
		return 0;
	v2 e = normalize( sub( p2, p1 ) );
	v2 right[P_MAX_POLY];
	int rightCount = 0;
	int bestIndex = 0;
	float bestDistance = cross( sub( ps[bestIndex], p1 ), e );
	if ( bestDistance > 0.0f )
		right[rightCount++] = ps[bestIndex];
	for ( int i = 1; i < count; ++i )
	{
		float d = cross( sub( ps[i], p1 ), e );
		if ( d > bestDistance )
		{
			bestIndex = i;
			bestDistance = d;
		}
		if ( d > 0.0f )
			right[rightCount++] = ps[i];
	}
	if ( bestDistance < 2.0f * P_LINEAR_SLOP )
		return 0;
	v2 best = ps[bestIndex];
	v2 h1[P_MAX_POLY], h2[P_MAX_POLY];
	int n1 = hull_recurse( p1, best, right, rightCount, h1 );
	int n2 = hull_recurse( best, p2, right, rightCount, h2 );
	int n = 0;
	for ( int i = 0; i < n1; ++i )
		out[n++] = h1[i];
	out[n++] = best;
	for ( int i = 0; i < n2; ++i )
		out[n++] = h2[i];
	return n;
}

// hull.c:76-233: welding, extreme points, quickhull, collinear merge.
// Returns the hull point count (0 when degenerate).
int p_compute_hull( const v2* points, int count, v2* hull )
{
	if ( count < 3 || count > P_MAX_POLY )
		return 0;
	box2 aabb = { { FLT_MAX, FLT_MAX }, { -FLT_MAX, -FLT_MAX } };
	v2 ps[P_MAX_POLY];
	int n = 0;
	const float tolSqr = 16.0f * P_LINEAR_SLOP * P_LINEAR_SLOP;
	for ( int i = 0; i < count; ++i )
	{
		aabb.lo = vmin( aabb.lo, points[i] );
		aabb.hi = vmax( aabb.hi, points[i] );
		v2 vi = points[i];
		bool unique = true;
		for ( int j = 0; j < i; ++j )
		{
			if ( distSq( vi, points[j] ) < tolSqr )
			{
				unique = false;
				break;
			}
		}
		if ( unique )
			ps[n++] = vi;
	}
	if ( n < 3 )
		return 0;
	v2 c = V( 0.5f * ( aabb.lo.x + aabb.hi.x ), 0.5f * ( aabb.lo.y + aabb.hi.y ) );
	int f1 = 0;
	float dsq1 = distSq( c, ps[f1] );
	for ( int i = 1; i < n; ++i )
	{
		float dsq = distSq( c, ps[i] );
		if ( dsq > dsq1 )
		{
			f1 = i;
			dsq1 = dsq;
		}
	}
	v2 p1 = ps[f1];
	ps[f1] = ps[n - 1];
	n = n - 1;
	int f2 = 0;
	float dsq2 = distSq( p1, ps[f2] );
	for ( int i = 1; i < n; ++i )
	{
		float dsq = distSq( p1, ps[i] );
		if ( dsq > dsq2 )
		{
			f2 = i;
			dsq2 = dsq;
		}
	}
	v2 p2 = ps[f2];
	ps[f2] = ps[n - 1];
	n = n - 1;
	v2 rightPts[P_MAX_POLY], leftPts[P_MAX_POLY];
	int rc = 0, lc = 0;
	v2 e = normalize( sub( p2, p1 ) );
	for ( int i = 0; i < n; ++i )
	{
		float d = cross( sub( ps[i], p1 ), e );
		if ( d >= 2.0f * P_LINEAR_SLOP )
			rightPts[rc++] = ps[i];
		else if ( d <= -2.0f * P_LINEAR_SLOP )
			leftPts[lc++] = ps[i];
	}
	v2 h1[P_MAX_POLY], h2[P_MAX_POLY];
	int n1 = hull_recurse( p1, p2, rightPts, rc, h1 );
	int n2 = hull_recurse( p2, p1, leftPts, lc, h2 );
	if ( n1 == 0 && n2 == 0 )
		return 0;
	int hc = 0;
	hull[hc++] = p1;
	for ( int i = 0; i < n1; ++i )
		hull[hc++] = h1[i];
	hull[hc++] = p2;
	for ( int i = 0; i < n2; ++i )
		hull[hc++] = h2[i];
	bool searching = true;
	while ( searching && hc > 2 )
	{
		searching = false;
		for ( int i = 0; i < hc; ++i )
		{
			int i1 = i;
			int i2 = ( i + 1 ) % hc;
			int i3 = ( i + 2 ) % hc;
			v2 r = normalize( sub( hull[i3], hull[i1] ) );
			float distance = cross( sub( hull[i2], hull[i1] ), r );
			if ( distance <= 2.0f * P_LINEAR_SLOP )
			{
				for ( int j = i2; j < hc - 1; ++j )
					hull[j] = hull[j + 1];
				hc -= 1;
				searching = true;
				break;
			}
		}
	}
	if ( hc < 3 )
		hc = 0;
	return hc;
}

// geometry.c:19-50
static v2 polygon_centroid( const v2* vertices, int count )
{
	v2 center = { 0.0f, 0.0f };
	float area = 0.0f;
	v2 origin = vertices[0];
	const float inv3 = 1.0f / 3.0f;
	for ( int i = 1; i < count - 1; ++i )
	{
		v2 e1 = sub( vertices[i], origin );
		v2 e2 = sub( vertices[i + 1], origin );
		float a = 0.5f * cross( e1, e2 );
		center = mulAdd( center, a * inv3, add( e1, e2 ) );
		area += a;
	}
	float invArea = 1.0f / area;
	center.x *= invArea;
	center.y *= invArea;
	return add( origin, center );
}

// geometry.c:52-83 (b2MakePolygon)
Polygon p_make_polygon( const v2* hull, int count, float radius )
{
	Polygon p = { 0 };
	p.count = count;
	p.radius = radius;
	for ( int i = 0; i < count; ++i )
		p.vertices[i] = hull[i];
	for ( int i = 0; i < count; ++i )
	{
		int i2 = i + 1 < count ? i + 1 : 0;
		v2 edge = sub( p.vertices[i2], p.vertices[i] );
		p.normals[i] = normalize( crossVS( edge, 1.0f ) );
	}
	p.centroid = polygon_centroid( p.vertices, count );
	return p;
}

// geometry.c:185-203 (b2MakeOffsetRoundedBox)
Polygon p_make_offset_rounded_box( float hx, float hy, v2 center, rot q, float radius )
{
	xform xf = { center, q };
	Polygon p = { 0 };
	p.count = 4;
	p.vertices[0] = xfPoint( xf, V( -hx, -hy ) );
	p.vertices[1] = xfPoint( xf, V( hx, -hy ) );
	p.vertices[2] = xfPoint( xf, V( hx, hy ) );
	p.vertices[3] = xfPoint( xf, V( -hx, hy ) );
	p.normals[0] = rotate( xf.q, V( 0.0f, -1.0f ) );
	p.normals[1] = rotate( xf.q, V( 1.0f, 0.0f ) );
	p.normals[2] = rotate( xf.q, V( 0.0f, 1.0f ) );
	p.normals[3] = rotate( xf.q, V( -1.0f, 0.0f ) );
	p.radius = radius;
	p.centroid = xf.p;
	return p;
}

// geometry.c:219-227
static MassData circle_mass( v2 center, float radius, float density )
{
	float rr = radius * radius;
	MassData m;
	m.mass = density * P_PI * rr;
	m.center = center;
	m.rotationalInertia = m.mass * ( 0.5f * rr + dot( center, center ) );
	return m;
}

// geometry.c:229-266
static MassData capsule_mass( v2 p1, v2 p2, float radius, float density )
{
	float rr = radius * radius;
	float len = length( sub( p2, p1 ) );
	float ll = len * len;
	float circleMass = density * ( P_PI * radius * radius );
	float boxMass = density * ( 2.0f * radius * len );
	MassData m;
	m.mass = circleMass + boxMass;
	m.center.x = 0.5f * ( p1.x + p2.x );
	m.center.y = 0.5f * ( p1.y + p2.y );
	float lc = 4.0f * radius / ( 3.0f * P_PI );
	float h = 0.5f * len;
	float circleInertia = circleMass * ( 0.5f * rr + h * h + 2.0f * h * lc );
	float boxInertia = boxMass * ( 4.0f * rr + ll ) / 12.0f;
	m.rotationalInertia = circleInertia + boxInertia;
	m.rotationalInertia += m.mass * dot( m.center, m.center );
	return m;
}

// geometry.c:268-364 (b2ComputePolygonMass)
static MassData polygon_mass( const Polygon* p, float density )
{
	if ( p->count == 1 )
		return circle_mass( p->vertices[0], p->radius, density );
	if ( p->count == 2 )
		return capsule_mass( p->vertices[0], p->vertices[1], p->radius, density );
	v2 vs[P_MAX_POLY] = { 0 };
	int count = p->count;
	float radius = p->radius;
	if ( radius > 0.0f )
	{
		float sqrt2 = 1.412f;
		for ( int i = 0; i < count; ++i )
		{
			int j = i == 0 ? count - 1 : i - 1;
			v2 mid = normalize( add( p->normals[j], p->normals[i] ) );
			vs[i] = mulAdd( p->vertices[i], sqrt2 * radius, mid );
		}
	}
	else
	{
		for ( int i = 0; i < count; ++i )
			vs[i] = p->vertices[i];
	}
	v2 center = { 0.0f, 0.0f };
	float area = 0.0f;
	float rotationalInertia = 0.0f;
	v2 r = vs[0];
	const float inv3 = 1.0f / 3.0f;
	for ( int i = 1; i < count - 1; ++i )
	{
		v2 e1 = sub( vs[i], r );
		v2 e2 = sub( vs[i + 1], r );
		float D = cross( e1, e2 );
		float triangleArea = 0.5f * D;
		area += triangleArea;
		center = mulAdd( center, triangleArea * inv3, add( e1, e2 ) );
		float ex1 = e1.x, ey1 = e1.y;
		float ex2 = e2.x, ey2 = e2.y;
		float intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
		float inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
		rotationalInertia += ( 0.25f * inv3 * D ) * ( intx2 + inty2 );
	}
	MassData m;
	m.mass = density * area;
	float invArea = 1.0f / area;
	center.x *= invArea;
	center.y *= invArea;
	m.center = add( r, center );
	m.rotationalInertia = density * rotationalInertia;
	m.rotationalInertia += m.mass * ( dot( m.center, m.center ) - dot( center, center ) );
	return m;
}

// shape.c:700-718 (b2ComputeShapeMass)
MassData p_shape_mass( const Shape* s )
{
	MassData zero = { 0 };
	switch ( s->g.type )
	{
		case SHAPE_CAPSULE:
			return capsule_mass( s->g.c1, s->g.c2, s->g.radius, s->density );
		case SHAPE_CIRCLE:
			return circle_mass( s->g.c1, s->g.radius, s->density );
		case SHAPE_POLYGON:
			return polygon_mass( &s->g.poly, s->density );
		default:
			return zero;
	}
}

// geometry.c:401-455 + shape.c:578-600 (b2ComputeShapeAABB)
box2 p_shape_aabb( const Geometry* g, xform xf )
{
	box2 b;
	switch ( g->type )
	{
		case SHAPE_CIRCLE:
		{
			v2 p = xfPoint( xf, g->c1 );
			float r = g->radius;
			b.lo = V( p.x - r, p.y - r );
			b.hi = V( p.x + r, p.y + r );
			return b;
		}
		case SHAPE_CAPSULE:
		{
			v2 v1 = xfPoint( xf, g->c1 );
			v2 v2p = xfPoint( xf, g->c2 );
			v2 r = { g->radius, g->radius };
			b.lo = sub( vmin( v1, v2p ), r );
			b.hi = add( vmax( v1, v2p ), r );
			return b;
		}
		case SHAPE_POLYGON:
		{
			const Polygon* p = &g->poly;
			v2 lo = xfPoint( xf, p->vertices[0] );
			v2 hi = lo;
			for ( int i = 1; i < p->count; ++i )
			{
				v2 v = xfPoint( xf, p->vertices[i] );
				lo = vmin( lo, v );
				hi = vmax( hi, v );
			}
			v2 r = { p->radius, p->radius };
			b.lo = sub( lo, r );
			b.hi = add( hi, r );
			return b;
		}
		case SHAPE_SEGMENT:
		default:
		{
			v2 v1 = xfPoint( xf, g->c1 );
			v2 v2p = xfPoint( xf, g->c2 );
			b.lo = vmin( v1, v2p );
			b.hi = vmax( v1, v2p );
			return b;
		}
	}
}

// shape.c:602-620 (b2GetShapeCentroid)
v2 p_shape_centroid( const Geometry* g )
{
	switch ( g->type )
	{
		case SHAPE_CAPSULE:
			return lerp( g->c1, g->c2, 0.5f );
		case SHAPE_CIRCLE:
			return g->c1;
		case SHAPE_POLYGON:
			return g->poly.centroid;
		case SHAPE_SEGMENT:
		case SHAPE_CHAIN_SEGMENT:
			return lerp( g->c1, g->c2, 0.5f );
		default:
			return V( 0.0f, 0.0f );
	}
}

// shape.c:720-790 (b2ComputeShapeExtent)
void p_shape_extent( const Shape* s, v2 localCenter, float* minExtent, float* maxExtent )
{
	const Geometry* g = &s->g;
	switch ( g->type )
	{
		case SHAPE_CAPSULE:
		{
			float radius = g->radius;
			*minExtent = radius;
			v2 c1 = sub( g->c1, localCenter );
			v2 c2 = sub( g->c2, localCenter );
			*maxExtent = sqrtf( fmaxp( lengthSq( c1 ), lengthSq( c2 ) ) ) + radius;
			return;
		}
		case SHAPE_CIRCLE:
		{
			float radius = g->radius;
			*minExtent = radius;
			*maxExtent = length( sub( g->c1, localCenter ) ) + radius;
			return;
		}
		case SHAPE_POLYGON:
		{
			const Polygon* p = &g->poly;
			float mn = P_HUGE;
			float mxSq = 0.0f;
			for ( int i = 0; i < p->count; ++i )
			{
				v2 v = p->vertices[i];
				float planeOffset = dot( p->normals[i], sub( v, p->centroid ) );
				mn = fminp( mn, planeOffset );
				float d = lengthSq( sub( v, localCenter ) );
				mxSq = fmaxp( mxSq, d );
			}
			*minExtent = mn + p->radius;
			*maxExtent = sqrtf( mxSq ) + p->radius;
			return;
		}
		case SHAPE_SEGMENT:
		default:
		{
			*minExtent = 0.0f;
			v2 c1 = sub( g->c1, localCenter );
			v2 c2 = sub( g->c2, localCenter );
			*maxExtent = sqrtf( fmaxp( lengthSq( c1 ), lengthSq( c2 ) ) );
			return;
		}
	}
}

// shape.h:104-117 (b2GetShapeRadius)
float p_shape_radius( const Geometry* g )
{
	switch ( g->type )
	{
		case SHAPE_CAPSULE:
			return g->radius;
		case SHAPE_CIRCLE:
			return g->radius;
		case SHAPE_POLYGON:
			return g->poly.radius;
		default:
			return 0.0f;
	}
}
