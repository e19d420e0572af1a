// Flattened definition records shared by the two CPU oracles (the reference
// harness oracle/ref_harness.c and the restatement oracle/port/). TEST
// INFRASTRUCTURE ONLY. The product's C-ABI (include/forge2d_gb300.h) declares
// records with the same field order so one Python scene builder can drive all
// three; this header is never included by product code.
//
// Field meaning follows forge2d's RawBox2D seam: RawBox2D.createWorld
// (packages/forge2d/lib/src/backend/raw_box2d.dart:18-29), createBody (:71-91)
// and RawShapeDef (raw_box2d_ffi.dart:564-584 shows the b2ShapeDef mapping).
#pragma once

#include <stdint.h>

typedef struct f2d_world_def
{
	double gravityX, gravityY;
	double restitutionThreshold;
	double hitEventThreshold;
	double contactHertz;
	double contactDampingRatio;
	double maxContactPushSpeed;
	double maximumLinearSpeed;
	int32_t enableSleep;
	int32_t enableContinuous;
} f2d_world_def;

typedef struct f2d_body_def
{
	int32_t type; // 0 static, 1 kinematic, 2 dynamic (b2BodyType)
	int32_t pad0;
	double positionX, positionY;
	double rotationCos, rotationSin;
	double linearVelocityX, linearVelocityY;
	double angularVelocity;
	double linearDamping;
	double angularDamping;
	double gravityScale;
	double sleepThreshold;
	int32_t enableSleep;
	int32_t isAwake;
	int32_t fixedRotation;
	int32_t isBullet;
	int32_t isEnabled;
	int32_t allowFastRotation;
} f2d_body_def;

typedef struct f2d_shape_def
{
	double friction;
	double restitution;
	double rollingResistance;
	double tangentSpeed;
	double density;
	int64_t categoryBits;
	int64_t maskBits;
	int32_t groupIndex;
	int32_t userMaterialId;
	int32_t isSensor;
	int32_t enableSensorEvents;
	int32_t enableContactEvents;
	int32_t enableHitEvents;
	int32_t enablePreSolveEvents;
	int32_t invokeContactCreation;
	int32_t updateBodyMass;
	int32_t pad0;
} f2d_shape_def;

typedef struct f2d_revolute_def
{
	int32_t bodyA, bodyB; // 0-based body ids
	double localAnchorAX, localAnchorAY;
	double localAnchorBX, localAnchorBY;
	double referenceAngle;
	double targetAngle;
	int32_t enableSpring;
	int32_t pad0;
	double hertz;
	double dampingRatio;
	int32_t enableLimit;
	int32_t pad1;
	double lowerAngle, upperAngle;
	int32_t enableMotor;
	int32_t pad2;
	double maxMotorTorque;
	double motorSpeed;
	double drawSize;
	int32_t collideConnected;
	int32_t pad3;
} f2d_revolute_def;

// Joints other than revolute, one definition for every type (fields a type
// does not use are ignored): b2WeldJointDef, b2DistanceJointDef,
// b2PrismaticJointDef, b2WheelJointDef, b2MotorJointDef, b2MouseJointDef,
// b2FilterJointDef (types.h:530-780).
#define F2D_JOINT_REVOLUTE 1
#define F2D_JOINT_WELD 2
#define F2D_JOINT_DISTANCE 3
#define F2D_JOINT_PRISMATIC 4
#define F2D_JOINT_WHEEL 5
#define F2D_JOINT_MOTOR 6
#define F2D_JOINT_MOUSE 7
#define F2D_JOINT_FILTER 8

typedef struct f2d_joint_def
{
	int32_t type;
	int32_t bodyA, bodyB; // 0-based body ids
	int32_t collideConnected;
	double localAnchorAX, localAnchorAY;
	double localAnchorBX, localAnchorBY;
	double referenceAngle;
	// weld
	double linearHertz, linearDampingRatio;
	double angularHertz, angularDampingRatio;
	// distance
	double length, minLength, maxLength;
	double hertz, dampingRatio;
	double maxMotorForce, motorSpeed;
	int32_t enableSpring, enableLimit, enableMotor, pad0;
	// prismatic and wheel
	double localAxisAX, localAxisAY;
	double targetTranslation, lowerTranslation, upperTranslation;
	double maxMotorTorque;
	// motor (maxForce also the mouse joint's)
	double linearOffsetX, linearOffsetY, angularOffset;
	double maxForce, maxTorque, correctionFactor;
	// mouse
	double targetX, targetY;
} f2d_joint_def;

// Callbacks (types.h b2CustomFilterFcn, b2PreSolveFcn) with 0-based shape ids:
// nonzero lets the pair collide / keeps the contact touching this step. The
// pre-solve view holds the new manifold before its anchors are shifted to
// the centres of mass (contact.c:504-517).
typedef struct f2d_manifold_point_view
{
	float pointX, pointY, anchorAX, anchorAY, anchorBX, anchorBY, separation;
	int32_t id;
} f2d_manifold_point_view;

typedef struct f2d_manifold_view
{
	float normalX, normalY;
	int32_t pointCount, pad0;
	f2d_manifold_point_view points[2];
} f2d_manifold_view;

typedef int32_t ( *orc_custom_filter_fn )( int32_t shapeA, int32_t shapeB, void* context );
typedef int32_t ( *orc_pre_solve_fn )( int32_t shapeA, int32_t shapeB, const f2d_manifold_view* manifold,
									   void* context );

// b2CastResultFcn with a 0-based shape id: returns -1 to ignore the hit, 0 to
// stop, a fraction to clip the ray, 1 to go on
typedef float ( *orc_cast_fn )( int32_t shape, float pointX, float pointY, float normalX, float normalY,
								float fraction, void* context );

// Dump strides used by the ref_get_* / orc_get_* state readers.
#define F2D_BODY_DUMP_STRIDE 12
#define F2D_CONTACT_DUMP_INTS 9
#define F2D_CONTACT_DUMP_FLOATS 25
