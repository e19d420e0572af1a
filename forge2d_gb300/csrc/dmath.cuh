// Device float math for the world step.
//
// Every operation is written as separate IEEE multiplies and adds in the
// operand order of Box2D v3.1.1's inline algebra (include/box2d/math_functions.h)
// and of its solver lanes (src/contact_solver.c), so that with -fmad=false the
// kernels produce the same bits as the reference's C code. Division and sqrtf
// use CUDA's correctly rounded defaults (no fast-math).
#pragma once

#include <cfloat>
#include <cstdint>

#define F2D_PI 3.14159265359f
#define F2D_LINEAR_SLOP 0.005f
#define F2D_SPECULATIVE ( 4.0f * F2D_LINEAR_SLOP )
#define F2D_AABB_MARGIN 0.05f
#define F2D_HUGE 100000.0f
#define F2D_MAX_ROTATION ( 0.25f * F2D_PI )
#define F2D_MAX_POLY 8
#define F2D_COLORS 12
#define F2D_OVERFLOW 11
#define F2D_NULL ( -1 )

#define HD __host__ __device__ __forceinline__

struct fv2
{
	float x, y;
};
struct frot
{
	float c, s;
};
struct fxf
{
	fv2 p;
	frot q;
};
struct fbox
{
	fv2 lo, hi;
};

// bit casts usable from host and device code
HD float bits_to_float( int i )
{
#ifdef __CUDA_ARCH__
	return __int_as_float( i );
#else
	float f;
	__builtin_memcpy( &f, &i, sizeof( f ) );
	return f;
#endif
}
HD int float_to_bits( float f )
{
#ifdef __CUDA_ARCH__
	return __float_as_int( f );
#else
	int i;
	__builtin_memcpy( &i, &f, sizeof( i ) );
	return i;
#endif
}

HD fv2 mk( float x, float y )
{
	fv2 r;
	r.x = x;
	r.y = y;
	return r;
}
HD float fmin_s( float a, float b )
{
	return a < b ? a : b;
}
HD float fmax_s( float a, float b )
{
	return a > b ? a : b;
}
HD float fabs_s( float a )
{
	return a < 0 ? -a : a;
}
HD float fclamp_s( float a, float lo, float hi )
{
	return a < lo ? lo : ( a > hi ? hi : a );
}
HD float vdot( fv2 a, fv2 b )
{
	return a.x * b.x + a.y * b.y;
}
HD float vcross( fv2 a, fv2 b )
{
	return a.x * b.y - a.y * b.x;
}
HD fv2 vcrossVS( fv2 v, float s )
{
	return mk( s * v.y, -s * v.x );
}
HD fv2 vcrossSV( float s, fv2 v )
{
	return mk( -s * v.y, s * v.x );
}
HD fv2 vleft( fv2 v )
{
	return mk( -v.y, v.x );
}
HD fv2 vright( fv2 v )
{
	return mk( v.y, -v.x );
}
HD fv2 vadd( fv2 a, fv2 b )
{
	return mk( a.x + b.x, a.y + b.y );
}
HD fv2 vsub( fv2 a, fv2 b )
{
	return mk( a.x - b.x, a.y - b.y );
}
HD fv2 vneg( fv2 a )
{
	return mk( -a.x, -a.y );
}
HD fv2 vlerp( fv2 a, fv2 b, float t )
{
	return mk( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y );
}
HD fv2 vscale( float s, fv2 v )
{
	return mk( s * v.x, s * v.y );
}
HD fv2 vmuladd( fv2 a, float s, fv2 b )
{
	return mk( a.x + s * b.x, a.y + s * b.y );
}
HD fv2 vmulsub( fv2 a, float s, fv2 b )
{
	return mk( a.x - s * b.x, a.y - s * b.y );
}
HD fv2 vmin2( fv2 a, fv2 b )
{
	return mk( fmin_s( a.x, b.x ), fmin_s( a.y, b.y ) );
}
HD fv2 vmax2( fv2 a, fv2 b )
{
	return mk( fmax_s( a.x, b.x ), fmax_s( a.y, b.y ) );
}
HD float vlen( fv2 v )
{
	return sqrtf( v.x * v.x + v.y * v.y );
}
HD float vlen2( fv2 v )
{
	return v.x * v.x + v.y * v.y;
}
HD float vdist2( fv2 a, fv2 b )
{
	float cx = b.x - a.x, cy = b.y - a.y;
	return cx * cx + cy * cy;
}
HD fv2 vnormalize( fv2 v )
{
	float len = sqrtf( v.x * v.x + v.y * v.y );
	if ( len < FLT_EPSILON )
		return mk( 0.0f, 0.0f );
	float inv = 1.0f / len;
	return mk( inv * v.x, inv * v.y );
}
HD fv2 vlen_norm( float* len, fv2 v )
{
	*len = sqrtf( v.x * v.x + v.y * v.y );
	if ( *len < FLT_EPSILON )
		return mk( 0.0f, 0.0f );
	float inv = 1.0f / *len;
	return mk( inv * v.x, inv * v.y );
}
HD frot rnormalize( frot q )
{
	float mag = sqrtf( q.s * q.s + q.c * q.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	frot r;
	r.c = q.c * inv;
	r.s = q.s * inv;
	return r;
}
HD frot rintegrate( frot q1, float da )
{
	frot q2;
	q2.c = q1.c - da * q1.s;
	q2.s = q1.s + da * q1.c;
	float mag = sqrtf( q2.s * q2.s + q2.c * q2.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	frot r;
	r.c = q2.c * inv;
	r.s = q2.s * inv;
	return r;
}
HD frot rnlerp( frot q1, frot q2, float t )
{
	float omt = 1.0f - t;
	frot q;
	q.c = omt * q1.c + t * q2.c;
	q.s = omt * q1.s + t * q2.s;
	return rnormalize( q );
}
HD frot rmul( frot q, frot r )
{
	frot o;
	o.s = q.s * r.c + q.c * r.s;
	o.c = q.c * r.c - q.s * r.s;
	return o;
}
HD frot rinvmul( frot q, frot r )
{
	frot o;
	o.s = q.c * r.s - q.s * r.c;
	o.c = q.c * r.c + q.s * r.s;
	return o;
}
HD fv2 rrot( frot q, fv2 v )
{
	return mk( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y );
}
HD fv2 rinvrot( frot q, fv2 v )
{
	return mk( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y );
}
HD fv2 xpoint( fxf t, fv2 p )
{
	float x = ( t.q.c * p.x - t.q.s * p.y ) + t.p.x;
	float y = ( t.q.s * p.x + t.q.c * p.y ) + t.p.y;
	return mk( x, y );
}
HD fxf xinvmul( fxf A, fxf B )
{
	fxf C;
	C.q = rinvmul( A.q, B.q );
	C.p = rinvrot( A.q, vsub( B.p, A.p ) );
	return C;
}
HD bool box_contains( fbox a, fbox b )
{
	bool s = true;
	s = s && a.lo.x <= b.lo.x;
	s = s && a.lo.y <= b.lo.y;
	s = s && b.hi.x <= a.hi.x;
	s = s && b.hi.y <= a.hi.y;
	return s;
}
HD bool box_overlaps( fbox a, fbox b )
{
	return !( b.lo.x > a.hi.x || b.lo.y > a.hi.y || a.lo.x > b.hi.x || a.lo.y > b.hi.y );
}
HD fbox box_union( fbox a, fbox b )
{
	fbox c;
	c.lo.x = fmin_s( a.lo.x, b.lo.x );
	c.lo.y = fmin_s( a.lo.y, b.lo.y );
	c.hi.x = fmax_s( a.hi.x, b.hi.x );
	c.hi.y = fmax_s( a.hi.y, b.hi.y );
	return c;
}
HD fbox box_from4( float4 f )
{
	fbox b;
	b.lo.x = f.x;
	b.lo.y = f.y;
	b.hi.x = f.z;
	b.hi.y = f.w;
	return b;
}
HD float4 box_to4( fbox b )
{
	return make_float4( b.lo.x, b.lo.y, b.hi.x, b.hi.y );
}
HD fbox box_grow( fbox b, float m )
{
	fbox r;
	r.lo.x = b.lo.x - m;
	r.lo.y = b.lo.y - m;
	r.hi.x = b.hi.x + m;
	r.hi.y = b.hi.y + m;
	return r;
}
HD fv2 solve22( fv2 cx, fv2 cy, fv2 b )
{
	float a11 = cx.x, a12 = cy.x, a21 = cx.y, a22 = cy.y;
	float det = a11 * a22 - a12 * a21;
	if ( det != 0.0f )
		det = 1.0f / det;
	return mk( det * ( a22 * b.x - a12 * b.y ), det * ( a11 * b.y - a21 * b.x ) );
}

// math_functions.c:61-102 minimax atan2 (operand order kept)
// math_functions.h:541-565 b2MulMV, b2GetInverse22 (matrix by columns cx, cy)
HD fv2 mulMV( fv2 cx, fv2 cy, fv2 v )
{
	return mk( cx.x * v.x + cy.x * v.y, cx.y * v.x + cy.y * v.y );
}
HD float4 inverse22( fv2 cx, fv2 cy )
{
	float a = cx.x, b = cy.x, c = cx.y, d = cy.y;
	float det = a * d - b * c;
	if ( det != 0.0f )
		det = 1.0f / det;
	return make_float4( det * d, -det * c, -det * b, det * a );
}

HD float f2d_atan2( float y, float x )
{
	if ( x == 0.0f && y == 0.0f )
		return 0.0f;
	float ax = fabs_s( x );
	float ay = fabs_s( y );
	float mx = fmax_s( ay, ax );
	float mn = fmin_s( ay, ax );
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

HD float relative_angle( frot b, frot a )
{
	float s = b.s * a.c - b.c * a.s;
	float c = b.c * a.c + b.s * a.s;
	return f2d_atan2( s, c );
}

// b2MakeSoft (solver.h:140-180)
struct Soft
{
	float biasRate, massScale, impulseScale;
};

HD Soft make_soft( float hertz, float zeta, float h )
{
	Soft s;
	if ( hertz == 0.0f )
	{
		s.biasRate = 0.0f;
		s.massScale = 0.0f;
		s.impulseScale = 0.0f;
		return s;
	}
	float omega = 2.0f * F2D_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	s.biasRate = omega / a1;
	s.massScale = a2 * a3;
	s.impulseScale = a3;
	return s;
}
