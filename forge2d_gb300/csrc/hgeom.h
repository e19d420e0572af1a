// Host-side creation-path geometry: convex hull, polygon construction, mass
// properties, extents and AABBs. These run once per shape when a user
// creates it, exactly as in Box2D v3.1.1 (packages/forge2d/third_party/box2d/
// src/hull.c:12-233, geometry.c:19-455, shape.c:578-790), so that the GPU
// world starts from bit-identical rows. Compiled with -ffp-contract=off.
#pragma once

#include "dmath.cuh"
#include "dworld.cuh"

struct HPoly
{
	fv2 v[F2D_MAX_POLY];
	fv2 n[F2D_MAX_POLY];
	fv2 centroid;
	float radius;
	int count;
};

struct HShapeGeom
{
	int type; // ST_*
	fv2 c1, c2;
	float radius;
	HPoly poly;
	fv2 g1, g2; // chain segment ghost vertices (before c1, after c2)
};

struct HMass
{
	float mass;
	fv2 center;
	float rotationalInertia;
};

int h_compute_hull( const fv2* points, int count, fv2* hull );
HPoly h_make_polygon( const fv2* hull, int count, float radius );
HPoly h_make_offset_rounded_box( float hx, float hy, fv2 center, frot q, float radius );
HMass h_shape_mass( const HShapeGeom& g, float density );
fbox h_shape_aabb( const HShapeGeom& g, fxf xf );
fv2 h_shape_centroid( const HShapeGeom& g );
void h_shape_extent( const HShapeGeom& g, fv2 localCenter, float* minExtent, float* maxExtent );
bool h_raycast_shape( const HShapeGeom& g, fxf xf, fv2 origin, fv2 translation, float maxFraction, fv2* point,
					  fv2* normal, float* fraction );
