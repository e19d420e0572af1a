// Scalar float math of the restatement. TEST INFRASTRUCTURE (oracle).
// Restates the inline vector/rotation algebra of Box2D v3.1.1,
// include/box2d/math_functions.h:126-660, keeping each expression's operand
// order so the IEEE results are bit-identical when compiled with
// -ffp-contract=off. min/max keep the compare-select forms of
// math_functions.h:126-147 (a<b?a:b, a>b?a:b).
#pragma once

#include <float.h>
#include <math.h>
#include <stdbool.h>
#include <stdint.h>

#define P_PI 3.14159265359f
#define P_LINEAR_SLOP 0.005f
#define P_SPECULATIVE ( 4.0f * P_LINEAR_SLOP )
#define P_AABB_MARGIN 0.05f
#define P_HUGE 100000.0f
#define P_MAX_ROTATION ( 0.25f * P_PI )
#define P_TIME_TO_SLEEP 0.5f
#define P_MAX_POLY 8
#define P_COLORS 12
#define P_OVERFLOW 11
#define P_NULL -1

typedef struct v2
{
	float x, y;
} v2;
typedef struct rot
{
	float c, s;
} rot;
typedef struct xform
{
	v2 p;
	rot q;
} xform;
typedef struct box2
{
	v2 lo, hi;
} box2;

static inline float fminp( float a, float b )
{
	return a < b ? a : b;
}
static inline float fmaxp( float a, float b )
{
	return a > b ? a : b;
}
static inline float fabsp( float a )
{
	return a < 0 ? -a : a;
}
static inline float fclampp( float a, float lo, float hi )
{
	return a < lo ? lo : ( a > hi ? hi : a );
}
static inline int iminp( int a, int b )
{
	return a < b ? a : b;
}
static inline int imaxp( int a, int b )
{
	return a > b ? a : b;
}

static inline v2 V( float x, float y )
{
	v2 r = { x, y };
	return r;
}
static inline float dot( v2 a, v2 b )
{
	return a.x * b.x + a.y * b.y;
}
static inline float cross( v2 a, v2 b )
{
	return a.x * b.y - a.y * b.x;
}
static inline v2 crossVS( v2 v, float s )
{
	return V( s * v.y, -s * v.x );
}
static inline v2 crossSV( float s, v2 v )
{
	return V( -s * v.y, s * v.x );
}
static inline v2 leftPerp( v2 v )
{
	return V( -v.y, v.x );
}
static inline v2 rightPerp( v2 v )
{
	return V( v.y, -v.x );
}
static inline v2 add( v2 a, v2 b )
{
	return V( a.x + b.x, a.y + b.y );
}
static inline v2 sub( v2 a, v2 b )
{
	return V( a.x - b.x, a.y - b.y );
}
static inline v2 neg( v2 a )
{
	return V( -a.x, -a.y );
}
static inline v2 lerp( v2 a, v2 b, float t )
{
	return V( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y );
}
static inline v2 mulSV( float s, v2 v )
{
	return V( s * v.x, s * v.y );
}
static inline v2 mulAdd( v2 a, float s, v2 b )
{
	return V( a.x + s * b.x, a.y + s * b.y );
}
static inline v2 mulSub( v2 a, float s, v2 b )
{
	return V( a.x - s * b.x, a.y - s * b.y );
}
static inline v2 vmin( v2 a, v2 b )
{
	return V( fminp( a.x, b.x ), fminp( a.y, b.y ) );
}
static inline v2 vmax( v2 a, v2 b )
{
	return V( fmaxp( a.x, b.x ), fmaxp( a.y, b.y ) );
}
static inline float length( v2 v )
{
	return sqrtf( v.x * v.x + v.y * v.y );
}
static inline float lengthSq( v2 v )
{
	return v.x * v.x + v.y * v.y;
}
static inline float distSq( v2 a, v2 b )
{
	v2 c = { b.x - a.x, b.y - a.y };
	return c.x * c.x + c.y * c.y;
}
static inline v2 normalize( v2 v )
{
	float len = sqrtf( v.x * v.x + v.y * v.y );
	if ( len < FLT_EPSILON )
		return V( 0.0f, 0.0f );
	float inv = 1.0f / len;
	return V( inv * v.x, inv * v.y );
}
static inline v2 lengthAndNormalize( float* len, v2 v )
{
	*len = sqrtf( v.x * v.x + v.y * v.y );
	if ( *len < FLT_EPSILON )
		return V( 0.0f, 0.0f );
	float inv = 1.0f / *len;
	return V( inv * v.x, inv * v.y );
}
static inline rot normalizeRot( rot q )
{
	float mag = sqrtf( q.s * q.s + q.c * q.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	rot r = { q.c * inv, q.s * inv };
	return r;
}
static inline rot integrateRot( rot q1, float da )
{
	rot q2 = { q1.c - da * q1.s, q1.s + da * q1.c };
	float mag = sqrtf( q2.s * q2.s + q2.c * q2.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	rot r = { q2.c * inv, q2.s * inv };
	return r;
}
static inline rot nlerpRot( rot q1, rot q2, float t )
{
	float omt = 1.0f - t;
	rot q = { omt * q1.c + t * q2.c, omt * q1.s + t * q2.s };
	return normalizeRot( q );
}
static inline rot mulRot( rot q, rot r )
{
	rot o;
	o.s = q.s * r.c + q.c * r.s;
	o.c = q.c * r.c - q.s * r.s;
	return o;
}
static inline rot invMulRot( rot q, rot r )
{
	rot o;
	o.s = q.c * r.s - q.s * r.c;
	o.c = q.c * r.c + q.s * r.s;
	return o;
}
static inline v2 rotate( rot q, v2 v )
{
	return V( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y );
}
static inline v2 invRotate( rot q, v2 v )
{
	return V( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y );
}
static inline v2 xfPoint( xform t, v2 p )
{
	float x = ( t.q.c * p.x - t.q.s * p.y ) + t.p.x;
	float y = ( t.q.s * p.x + t.q.c * p.y ) + t.p.y;
	return V( x, y );
}
static inline v2 invXfPoint( xform t, v2 p )
{
	float vx = p.x - t.p.x;
	float vy = p.y - t.p.y;
	return V( t.q.c * vx + t.q.s * vy, -t.q.s * vx + t.q.c * vy );
}
static inline xform invMulXf( xform A, xform B )
{
	xform C;
	C.q = invMulRot( A.q, B.q );
	C.p = invRotate( A.q, sub( B.p, A.p ) );
	return C;
}
static inline bool boxContains( box2 a, box2 b )
{
	bool s = true;
	s = s && a.lo.x <= b.lo.x;
	s = s && a.lo.y <= b.lo.y;
	s = s && b.hi.x <= a.hi.x;
	s = s && b.hi.y <= a.hi.y;
	return s;
}
static inline bool boxOverlaps( box2 a, box2 b )
{
	return !( b.lo.x > a.hi.x || b.lo.y > a.hi.y || a.lo.x > b.hi.x || a.lo.y > b.hi.y );
}
static inline box2 boxUnion( box2 a, box2 b )
{
	box2 c;
	c.lo.x = fminp( a.lo.x, b.lo.x );
	c.lo.y = fminp( a.lo.y, b.lo.y );
	c.hi.x = fmaxp( a.hi.x, b.hi.x );
	c.hi.y = fmaxp( a.hi.y, b.hi.y );
	return c;
}
static inline v2 solve22( v2 cx, v2 cy, v2 b )
{
	float a11 = cx.x, a12 = cy.x, a21 = cx.y, a22 = cy.y;
	float det = a11 * a22 - a12 * a21;
	if ( det != 0.0f )
		det = 1.0f / det;
	return V( det * ( a22 * b.x - a12 * b.y ), det * ( a11 * b.y - a21 * b.x ) );
}

// math_functions.c:61-102 (minimax atan2) and :108-151 (Bhaskara cos/sin)
float p_atan2( float y, float x );
void p_cossin( float radians, float* c, float* s );
// math_functions.h:541-565 b2MulMV, b2GetInverse22 (columns cx, cy)
static inline v2 mulMV( v2 cx, v2 cy, v2 v )
{
	return V( cx.x * v.x + cy.x * v.y, cx.y * v.x + cy.y * v.y );
}

static inline void inverse22( v2 cx, v2 cy, v2* icx, v2* icy )
{
	float a = cx.x, b = cy.x, c = cx.y, d = cy.y;
	float det = a * d - b * c;
	if ( det != 0.0f )
		det = 1.0f / det;
	*icx = V( det * d, -det * c );
	*icy = V( -det * b, det * a );
}

static inline float relativeAngle( rot b, rot a )
{
	float s = b.s * a.c - b.c * a.s;
	float c = b.c * a.c + b.s * a.s;
	return p_atan2( s, c );
}
static inline float unwindAngle( float r )
{
	return remainderf( r, 2.0f * P_PI );
}
