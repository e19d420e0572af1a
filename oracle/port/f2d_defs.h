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

// property codes of the generic get/set calls (the same values as the
// product header's; a CPU test compares the two lists)
#define F2D_BODY_LINEAR_DAMPING 1
#define F2D_BODY_ANGULAR_DAMPING 2
#define F2D_BODY_GRAVITY_SCALE 3
#define F2D_BODY_BULLET 4
#define F2D_BODY_FIXED_ROTATION 5
#define F2D_BODY_ENABLED 6
#define F2D_BODY_TYPE 7
#define F2D_BODY_LOCAL_CENTER_X 8
#define F2D_BODY_LOCAL_CENTER_Y 9
#define F2D_BODY_WORLD_CENTER_X 10
#define F2D_BODY_WORLD_CENTER_Y 11
#define F2D_SHAPE_DENSITY 1
#define F2D_SHAPE_FRICTION 2
#define F2D_SHAPE_RESTITUTION 3
#define F2D_SHAPE_SENSOR 4
#define F2D_SHAPE_SENSOR_EVENTS 5
#define F2D_SHAPE_CONTACT_EVENTS 6
#define F2D_SHAPE_HIT_EVENTS 7
#define F2D_SHAPE_PRESOLVE_EVENTS 8
#define F2D_SHAPE_CATEGORY 9
#define F2D_SHAPE_MASK 10
#define F2D_SHAPE_GROUP 11
#define F2D_JP_TYPE 1
#define F2D_JP_LOCAL_ANCHOR_AX 2
#define F2D_JP_LOCAL_ANCHOR_AY 3
#define F2D_JP_LOCAL_ANCHOR_BX 4
#define F2D_JP_LOCAL_ANCHOR_BY 5
#define F2D_JP_SPRING_ENABLED 6
#define F2D_JP_SPRING_HERTZ 7
#define F2D_JP_SPRING_DAMPING 8
#define F2D_JP_TARGET 9
#define F2D_JP_LIMIT_ENABLED 10
#define F2D_JP_LOWER 11
#define F2D_JP_UPPER 12
#define F2D_JP_MOTOR_ENABLED 13
#define F2D_JP_MOTOR_SPEED 14
#define F2D_JP_MAX_MOTOR 15
#define F2D_JP_MOTOR_EFFORT 16
#define F2D_JP_LENGTH 17
#define F2D_JP_MIN_LENGTH 18
#define F2D_JP_MAX_LENGTH 19
#define F2D_JP_CURRENT 20
#define F2D_JP_SPEED 21
#define F2D_JP_LINEAR_HERTZ 22
#define F2D_JP_LINEAR_DAMPING 23
#define F2D_JP_ANGULAR_HERTZ 24
#define F2D_JP_ANGULAR_DAMPING 25
#define F2D_JP_LINEAR_OFFSET_X 26
#define F2D_JP_LINEAR_OFFSET_Y 27
#define F2D_JP_ANGULAR_OFFSET 28
#define F2D_JP_MAX_FORCE 29
#define F2D_JP_MAX_TORQUE 30
#define F2D_JP_CORRECTION 31
#define F2D_JP_TARGET_X 32
#define F2D_JP_TARGET_Y 33
