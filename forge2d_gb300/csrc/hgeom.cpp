// Host creation-path geometry; see hgeom.h. Each function follows the cited
// Box2D v3.1.1 function's arithmetic (packages/forge2d/third_party/box2d/src).
#include "hgeom.h"

#include <cmath>

static inline float slop()
{
	return F2D_LINEAR_SLOP;
}

// hull.c:12-71
static int hull_recurse( fv2 p1, fv2 p2, const fv2* ps, int count, fv2* out )
{
	if ( count == 0 )
		return 0;
	fv2 e = vnormalize( vsub( p2, p1 ) );
	fv2 right[F2D_MAX_POLY];
	int rightCount = 0;
	int bestIndex = 0;
	float bestDistance = vcross( vsub( ps[bestIndex], p1 ), e );
	if ( bestDistance > 0.0f )
		right[rightCount++] = ps[bestIndex];
	for ( int i = 1; i < count; ++i )
	{
		float d = vcross( vsub( ps[i], p1 ), e );
		if ( d > bestDistance )
		{
			bestIndex = i;
			bestDistance = d;
		}
		if ( d > 0.0f )
			right[rightCount++] = ps[i];
	}
	if ( bestDistance < 2.0f * slop() )
		return 0;
	fv2 best = ps[bestIndex];
	fv2 h1[F2D_MAX_POLY], h2[F2D_MAX_POLY];
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

// hull.c:76-233 (b2ComputeHull)
int h_compute_hull( const fv2* points, int count, fv2* hull )
{
	if ( count < 3 || count > F2D_MAX_POLY )
		return 0;
	fbox aabb;
	aabb.lo = mk( FLT_MAX, FLT_MAX );
	aabb.hi = mk( -FLT_MAX, -FLT_MAX );
	fv2 ps[F2D_MAX_POLY];
	int n = 0;
	const float tolSqr = 16.0f * slop() * slop();
	for ( int i = 0; i < count; ++i )
	{
		aabb.lo = vmin2( aabb.lo, points[i] );
		aabb.hi = vmax2( aabb.hi, points[i] );
		fv2 vi = points[i];
		bool unique = true;
		for ( int j = 0; j < i; ++j )
			if ( vdist2( vi, points[j] ) < tolSqr )
			{
				unique = false;
				break;
			}
		if ( unique )
			ps[n++] = vi;
	}
	if ( n < 3 )
		return 0;
	fv2 c = mk( 0.5f * ( aabb.lo.x + aabb.hi.x ), 0.5f * ( aabb.lo.y + aabb.hi.y ) );
	int f1 = 0;
	float dsq1 = vdist2( c, ps[f1] );
	for ( int i = 1; i < n; ++i )
	{
		float dsq = vdist2( c, ps[i] );
		if ( dsq > dsq1 )
		{
			f1 = i;
			dsq1 = dsq;
		}
	}
	fv2 p1 = ps[f1];
	ps[f1] = ps[n - 1];
	n = n - 1;
	int f2 = 0;
	float dsq2 = vdist2( p1, ps[f2] );
	for ( int i = 1; i < n; ++i )
	{
		float dsq = vdist2( p1, ps[i] );
		if ( dsq > dsq2 )
		{
			f2 = i;
			dsq2 = dsq;
		}
	}
	fv2 p2 = ps[f2];
	ps[f2] = ps[n - 1];
	n = n - 1;
	fv2 rightPts[F2D_MAX_POLY], leftPts[F2D_MAX_POLY];
	int rc = 0, lc = 0;
	fv2 e = vnormalize( vsub( p2, p1 ) );
	for ( int i = 0; i < n; ++i )
	{
		float d = vcross( vsub( ps[i], p1 ), e );
		if ( d >= 2.0f * slop() )
			rightPts[rc++] = ps[i];
		else if ( d <= -2.0f * slop() )
			leftPts[lc++] = ps[i];
	}
	fv2 h1[F2D_MAX_POLY], h2[F2D_MAX_POLY];
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
			int i1 = i, i2 = ( i + 1 ) % hc, i3 = ( i + 2 ) % hc;
			fv2 r = vnormalize( vsub( hull[i3], hull[i1] ) );
			float distance = vcross( vsub( hull[i2], hull[i1] ), r );
			if ( distance <= 2.0f * slop() )
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
static fv2 polygon_centroid( const fv2* v, int count )
{
	fv2 center = mk( 0.0f, 0.0f );
	float area = 0.0f;
	fv2 origin = v[0];
	const float inv3 = 1.0f / 3.0f;
	for ( int i = 1; i < count - 1; ++i )
	{
		fv2 e1 = vsub( v[i], origin );
		fv2 e2 = vsub( v[i + 1], origin );
		float a = 0.5f * vcross( e1, e2 );
		center = vmuladd( center, a * inv3, vadd( e1, e2 ) );
		area += a;
	}
	float invArea = 1.0f / area;
	center.x *= invArea;
	center.y *= invArea;
	return vadd( origin, center );
}

// geometry.c:52-83 (b2MakePolygon)
HPoly h_make_polygon( const fv2* hull, int count, float radius )
{
	HPoly p = {};
	p.count = count;
	p.radius = radius;
	for ( int i = 0; i < count; ++i )
		p.v[i] = hull[i];
	for ( int i = 0; i < count; ++i )
	{
		int i2 = i + 1 < count ? i + 1 : 0;
		fv2 edge = vsub( p.v[i2], p.v[i] );
		p.n[i] = vnormalize( vcrossVS( edge, 1.0f ) );
	}
	p.centroid = polygon_centroid( p.v, count );
	return p;
}

// geometry.c:185-203 (b2MakeOffsetRoundedBox)
HPoly h_make_offset_rounded_box( float hx, float hy, fv2 center, frot q, float radius )
{
	fxf xf;
	xf.p = center;
	xf.q = q;
	HPoly p = {};
	p.count = 4;
	p.v[0] = xpoint( xf, mk( -hx, -hy ) );
	p.v[1] = xpoint( xf, mk( hx, -hy ) );
	p.v[2] = xpoint( xf, mk( hx, hy ) );
	p.v[3] = xpoint( xf, mk( -hx, hy ) );
	p.n[0] = rrot( xf.q, mk( 0.0f, -1.0f ) );
	p.n[1] = rrot( xf.q, mk( 1.0f, 0.0f ) );
	p.n[2] = rrot( xf.q, mk( 0.0f, 1.0f ) );
	p.n[3] = rrot( xf.q, mk( -1.0f, 0.0f ) );
	p.radius = radius;
	p.centroid = xf.p;
	return p;
}

// geometry.c:219-227
static HMass circle_mass( fv2 center, float radius, float density )
{
	float rr = radius * radius;
	HMass m;
	m.mass = density * F2D_PI * rr;
	m.center = center;
	m.rotationalInertia = m.mass * ( 0.5f * rr + vdot( center, center ) );
	return m;
}

// geometry.c:229-266
static HMass capsule_mass( fv2 p1, fv2 p2, float radius, float density )
{
	float rr = radius * radius;
	float len = vlen( vsub( p2, p1 ) );
	float ll = len * len;
	float circleMass = density * ( F2D_PI * radius * radius );
	float boxMass = density * ( 2.0f * radius * len );
	HMass m;
	m.mass = circleMass + boxMass;
	m.center.x = 0.5f * ( p1.x + p2.x );
	m.center.y = 0.5f * ( p1.y + p2.y );
	float lc = 4.0f * radius / ( 3.0f * F2D_PI );
	float h = 0.5f * len;
	float circleInertia = circleMass * ( 0.5f * rr + h * h + 2.0f * h * lc );
	float boxInertia = boxMass * ( 4.0f * rr + ll ) / 12.0f;
	m.rotationalInertia = circleInertia + boxInertia;
	m.rotationalInertia += m.mass * vdot( m.center, m.center );
	return m;
}

// geometry.c:268-364
static HMass polygon_mass( const HPoly& p, float density )
{
	if ( p.count == 1 )
		return circle_mass( p.v[0], p.radius, density );
	if ( p.count == 2 )
		return capsule_mass( p.v[0], p.v[1], p.radius, density );
	fv2 vs[F2D_MAX_POLY] = {};
	int count = p.count;
	float radius = p.radius;
	if ( radius > 0.0f )
	{
		float sqrt2 = 1.412f;
		for ( int i = 0; i < count; ++i )
		{
			int j = i == 0 ? count - 1 : i - 1;
			fv2 mid = vnormalize( vadd( p.n[j], p.n[i] ) );
			vs[i] = vmuladd( p.v[i], sqrt2 * radius, mid );
		}
	}
	else
	{
		for ( int i = 0; i < count; ++i )
			vs[i] = p.v[i];
	}
	fv2 center = mk( 0.0f, 0.0f );
	float area = 0.0f;
	float rotationalInertia = 0.0f;
	fv2 r = vs[0];
	const float inv3 = 1.0f / 3.0f;
	for ( int i = 1; i < count - 1; ++i )
	{
		fv2 e1 = vsub( vs[i], r );
		fv2 e2 = vsub( vs[i + 1], r );
		float D = vcross( e1, e2 );
		float triangleArea = 0.5f * D;
		area += triangleArea;
		center = vmuladd( center, triangleArea * inv3, vadd( e1, e2 ) );
		float ex1 = e1.x, ey1 = e1.y;
		float ex2 = e2.x, ey2 = e2.y;
		float intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
		float inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
		rotationalInertia += ( 0.25f * inv3 * D ) * ( intx2 + inty2 );
	}
	HMass m;
	m.mass = density * area;
	float invArea = 1.0f / area;
	center.x *= invArea;
	center.y *= invArea;
	m.center = vadd( r, center );
	m.rotationalInertia = density * rotationalInertia;
	m.rotationalInertia += m.mass * ( vdot( m.center, m.center ) - vdot( center, center ) );
	return m;
}

HMass h_shape_mass( const HShapeGeom& g, float density )
{
	switch ( g.type )
	{
		case ST_CAPSULE:
			return capsule_mass( g.c1, g.c2, g.radius, density );
		case ST_CIRCLE:
			return circle_mass( g.c1, g.radius, density );
		case ST_POLYGON:
			return polygon_mass( g.poly, density );
		default:
		{
			HMass z = {};
			return z;
		}
	}
}

// geometry.c:401-455
fbox h_shape_aabb( const HShapeGeom& g, fxf xf )
{
	fbox b;
	switch ( g.type )
	{
		case ST_CIRCLE:
		{
			fv2 p = xpoint( xf, g.c1 );
			float r = g.radius;
			b.lo = mk( p.x - r, p.y - r );
			b.hi = mk( p.x + r, p.y + r );
			return b;
		}
		case ST_CAPSULE:
		{
			fv2 v1 = xpoint( xf, g.c1 );
			fv2 v2 = xpoint( xf, g.c2 );
			fv2 r = mk( g.radius, g.radius );
			b.lo = vsub( vmin2( v1, v2 ), r );
			b.hi = vadd( vmax2( v1, v2 ), r );
			return b;
		}
		case ST_POLYGON:
		{
			fv2 lo = xpoint( xf, g.poly.v[0] );
			fv2 hi = lo;
			for ( int i = 1; i < g.poly.count; ++i )
			{
				fv2 v = xpoint( xf, g.poly.v[i] );
				lo = vmin2( lo, v );
				hi = vmax2( hi, v );
			}
			fv2 r = mk( g.poly.radius, g.poly.radius );
			b.lo = vsub( lo, r );
			b.hi = vadd( hi, r );
			return b;
		}
		default:
		{
			fv2 v1 = xpoint( xf, g.c1 );
			fv2 v2 = xpoint( xf, g.c2 );
			b.lo = vmin2( v1, v2 );
			b.hi = vmax2( v1, v2 );
			return b;
		}
	}
}

// shape.c:602-620
fv2 h_shape_centroid( const HShapeGeom& g )
{
	switch ( g.type )
	{
		case ST_CAPSULE:
		case ST_SEGMENT:
		case ST_CHAIN:
			return vlerp( g.c1, g.c2, 0.5f );
		case ST_CIRCLE:
			return g.c1;
		case ST_POLYGON:
			return g.poly.centroid;
		default:
			return mk( 0.0f, 0.0f );
	}
}

// shape.c:720-790
void h_shape_extent( const HShapeGeom& g, fv2 localCenter, float* minExtent, float* maxExtent )
{
	switch ( g.type )
	{
		case ST_CAPSULE:
		{
			*minExtent = g.radius;
			fv2 c1 = vsub( g.c1, localCenter );
			fv2 c2 = vsub( g.c2, localCenter );
			*maxExtent = sqrtf( fmax_s( vlen2( c1 ), vlen2( c2 ) ) ) + g.radius;
			return;
		}
		case ST_CIRCLE:
			*minExtent = g.radius;
			*maxExtent = vlen( vsub( g.c1, localCenter ) ) + g.radius;
			return;
		case ST_POLYGON:
		{
			float mn = F2D_HUGE;
			float mxSq = 0.0f;
			for ( int i = 0; i < g.poly.count; ++i )
			{
				fv2 v = g.poly.v[i];
				float planeOffset = vdot( g.poly.n[i], vsub( v, g.poly.centroid ) );
				mn = fmin_s( mn, planeOffset );
				float d = vlen2( vsub( v, localCenter ) );
				mxSq = fmax_s( mxSq, d );
			}
			*minExtent = mn + g.poly.radius;
			*maxExtent = sqrtf( mxSq ) + g.poly.radius;
			return;
		}
		default:
		{
			*minExtent = 0.0f;
			fv2 c1 = vsub( g.c1, localCenter );
			fv2 c2 = vsub( g.c2, localCenter );
			*maxExtent = sqrtf( fmax_s( vlen2( c1 ), vlen2( c2 ) ) );
			return;
		}
	}
}
