/*
 * scenes.c -- seeded synthetic scene generators (see scenes.h).
 *
 * Scene layouts follow the reference benchmark and test scenes cited per function; the
 * sizes and distributions are the ones of the five benchmark workloads (small pyramid,
 * large pyramid with x jitter, tumbler with mixed shapes, batched uneven pyramids, box
 * drops with random velocity and friction).
 */
#include "scenes.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

void b2s_seed( b2sRandom* rng, uint64_t seed )
{
	/* PCG32 initialisation: the stream selector is derived from the seed. */
	rng->state = 0u;
	rng->inc = ( seed << 1u ) | 1u;
	b2s_next( rng );
	rng->state += 0x853c49e6748fea9bULL ^ seed;
	b2s_next( rng );
}

uint32_t b2s_next( b2sRandom* rng )
{
	uint64_t old = rng->state;
	rng->state = old * 6364136223846793005ULL + rng->inc;
	uint32_t xorshifted = (uint32_t)( ( ( old >> 18u ) ^ old ) >> 27u );
	uint32_t rot = (uint32_t)( old >> 59u );
	return ( xorshifted >> rot ) | ( xorshifted << ( ( 32u - rot ) & 31u ) );
}

float b2s_uniform( b2sRandom* rng, float lo, float hi )
{
	float u = (float)( b2s_next( rng ) >> 8 ) * ( 1.0f / 16777216.0f );
	return lo + ( hi - lo ) * u;
}

float b2s_normal( b2sRandom* rng )
{
	float sum = 0.0f;
	for ( int i = 0; i < 12; ++i )
		sum += b2s_uniform( rng, 0.0f, 1.0f );
	return sum - 6.0f;
}

b2WorldDef b2s_world_def( void )
{
	b2WorldDef def = b2DefaultWorldDef();
	def.enableSleep = false;
	def.enableContinous = true;
	return def;
}

static void b2s_ground( b2WorldId worldId, float friction )
{
	b2BodyDef bd = b2DefaultBodyDef();
	bd.position = ( b2Vec2 ){ 0.0f, -0.5f };
	b2BodyId groundId = b2CreateBody( worldId, &bd );
	b2Polygon box = b2MakeBox( 100.0f, 0.5f );
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.friction = friction;
	b2CreatePolygonShape( groundId, &sd, &box );
}

void b2s_add_pyramid( b2WorldId worldId, int baseCount, float jitter, uint64_t seed, float xOffset )
{
	b2sRandom rng;
	b2s_seed( &rng, seed );

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.enableSleep = false;

	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.6f;
	sd.restitution = 0.0f;

	float h = 0.5f;
	b2Polygon box = b2MakeSquare( h );
	float shift = 1.0f * h;

	for ( int i = 0; i < baseCount; ++i )
	{
		float y = ( 2.0f * i + 1.0f ) * shift;
		for ( int j = i; j < baseCount; ++j )
		{
			float x = ( i + 1.0f ) * shift + 2.0f * ( j - i ) * shift - h * baseCount;
			if ( jitter > 0.0f )
				x += b2s_uniform( &rng, -jitter, jitter );
			bd.position = ( b2Vec2 ){ x + xOffset, y };
			b2BodyId bodyId = b2CreateBody( worldId, &bd );
			b2CreatePolygonShape( bodyId, &sd, &box );
		}
	}
}

b2WorldId b2s_pyramid( int baseCount, float jitter, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;
	b2s_ground( worldId, 0.6f );
	b2s_add_pyramid( worldId, baseCount, jitter, seed, 0.0f );
	return worldId;
}

b2WorldId b2s_tumbler( int count, uint64_t seed, int variant )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;

	b2BodyDef gd = b2DefaultBodyDef();
	b2BodyId groundId = b2CreateBody( worldId, &gd );

	b2BodyDef td = b2DefaultBodyDef();
	td.type = b2_dynamicBody;
	td.position = ( b2Vec2 ){ 0.0f, 10.0f };
	b2BodyId tumblerId = b2CreateBody( worldId, &td );

	b2ShapeDef wallDef = b2DefaultShapeDef();
	wallDef.density = 50.0f;
	b2Polygon wall;
	wall = b2MakeOffsetBox( 0.5f, 10.0f, ( b2Vec2 ){ 10.0f, 0.0f }, 0.0f );
	b2CreatePolygonShape( tumblerId, &wallDef, &wall );
	wall = b2MakeOffsetBox( 0.5f, 10.0f, ( b2Vec2 ){ -10.0f, 0.0f }, 0.0f );
	b2CreatePolygonShape( tumblerId, &wallDef, &wall );
	wall = b2MakeOffsetBox( 10.0f, 0.5f, ( b2Vec2 ){ 0.0f, 10.0f }, 0.0f );
	b2CreatePolygonShape( tumblerId, &wallDef, &wall );
	wall = b2MakeOffsetBox( 10.0f, 0.5f, ( b2Vec2 ){ 0.0f, -10.0f }, 0.0f );
	b2CreatePolygonShape( tumblerId, &wallDef, &wall );

	b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
	jd.bodyIdA = groundId;
	jd.bodyIdB = tumblerId;
	jd.localAnchorA = ( b2Vec2 ){ 0.0f, 10.0f };
	jd.localAnchorB = ( b2Vec2 ){ 0.0f, 0.0f };
	jd.referenceAngle = 0.0f;
	jd.motorSpeed = variant == 1 ? ( b2_pi / 180.0f ) * 25.0f : 0.05f * b2_pi;
	jd.maxMotorTorque = 1e8f;
	jd.enableMotor = true;
	b2CreateRevoluteJoint( worldId, &jd );

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2ShapeDef sd = b2DefaultShapeDef();
	b2Polygon box = b2MakeBox( 0.125f, 0.125f );

	if ( variant == 1 )
	{
		int gridCount = 45;
		float y = -0.2f * gridCount + 10.0f;
		for ( int i = 0; i < gridCount; ++i )
		{
			float x = -0.2f * gridCount;
			for ( int j = 0; j < gridCount; ++j )
			{
				bd.position = ( b2Vec2 ){ x, y };
				b2BodyId bodyId = b2CreateBody( worldId, &bd );
				b2CreatePolygonShape( bodyId, &sd, &box );
				x += 0.4f;
			}
			y += 0.4f;
		}
		return worldId;
	}

	/* Jittered grid: the 19 x 19 m interior is cut into 45 x 45 cells, `count` distinct
	 * cells are drawn by a seeded shuffle and each body is placed uniformly inside the
	 * central part of its cell, which keeps shapes of size 0.25 from overlapping. */
	enum
	{
		gridN = 45
	};
	int cells[gridN * gridN];
	for ( int i = 0; i < gridN * gridN; ++i )
		cells[i] = i;
	b2sRandom rng;
	b2s_seed( &rng, seed );
	for ( int i = gridN * gridN - 1; i > 0; --i )
	{
		int j = (int)( b2s_next( &rng ) % (uint32_t)( i + 1 ) );
		int t = cells[i];
		cells[i] = cells[j];
		cells[j] = t;
	}

	if ( count > gridN * gridN )
		count = gridN * gridN;

	float cell = 19.0f / gridN;
	float slack = 0.5f * ( cell - 0.26f );
	b2Circle circle = { { 0.0f, 0.0f }, 0.125f };
	for ( int k = 0; k < count; ++k )
	{
		int ci = cells[k] % gridN;
		int cj = cells[k] / gridN;
		float cx = -9.5f + ( ci + 0.5f ) * cell;
		float cy = 0.5f + ( cj + 0.5f ) * cell;
		/* draws in statements of their own: the order of evaluation inside one
		 * initialiser list or argument list is unspecified */
		float jx = b2s_uniform( &rng, -slack, slack );
		float jy = b2s_uniform( &rng, -slack, slack );
		bd.position = ( b2Vec2 ){ cx + jx, cy + jy };
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
		if ( ( k & 1 ) == 0 )
			b2CreatePolygonShape( bodyId, &sd, &box );
		else
			b2CreateCircleShape( bodyId, &sd, &circle );
	}

	return worldId;
}

b2WorldId b2s_drop_boxes( int count, const float* heights, const float* vx, const float* vy, float friction )
{
	return b2s_drop_shapes( count, heights, vx, vy, friction, NULL );
}

b2WorldId b2s_drop_shapes( int count, const float* heights, const float* vx, const float* vy, float friction, const int* kinds )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;
	b2s_ground( worldId, friction );

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.enableSleep = false;
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = friction;
	b2Polygon box = b2MakeSquare( 0.5f );
	b2Circle circle = { { 0.0f, 0.0f }, 0.5f };
	b2Capsule capsule = { { -0.3f, 0.0f }, { 0.3f, 0.0f }, 0.25f };
	for ( int k = 0; k < count; ++k )
	{
		int kind = kinds != NULL ? kinds[k] : 0;
		/* a plank spans the whole row, under the bodies that follow it */
		float x = kind == 3 ? 0.75f * (float)( count - 1 ) : 1.5f * (float)k;
		bd.position = ( b2Vec2 ){ x, heights[k] };
		bd.linearVelocity = ( b2Vec2 ){ vx[k], vy[k] };
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
		if ( kind == 1 )
			b2CreateCircleShape( bodyId, &sd, &circle );
		else if ( kind == 2 )
			b2CreateCapsuleShape( bodyId, &sd, &capsule );
		else if ( kind == 3 )
		{
			b2Polygon plank = b2MakeBox( 0.75f * (float)count, 0.2f );
			b2CreatePolygonShape( bodyId, &sd, &plank );
		}
		else
			b2CreatePolygonShape( bodyId, &sd, &box );
	}
	return worldId;
}

void b2s_draw_ints( int n, uint64_t seed, int lo, int hi, int* out )
{
	b2sRandom rng;
	b2s_seed( &rng, seed );
	uint32_t span = (uint32_t)( hi - lo + 1 );
	for ( int i = 0; i < n; ++i )
		out[i] = lo + (int)( b2s_next( &rng ) % span );
}

void b2s_draw_uniform( int n, uint64_t seed, float lo, float hi, float* out )
{
	b2sRandom rng;
	b2s_seed( &rng, seed );
	for ( int i = 0; i < n; ++i )
		out[i] = b2s_uniform( &rng, lo, hi );
}

void b2s_draw_normal( int n, uint64_t seed, float* out )
{
	b2sRandom rng;
	b2s_seed( &rng, seed );
	for ( int i = 0; i < n; ++i )
		out[i] = b2s_normal( &rng );
}

b2WorldId b2s_hello_world( b2BodyId* bodyOut )
{
	b2WorldDef wd = b2DefaultWorldDef();
	wd.gravity = ( b2Vec2 ){ 0.0f, -10.0f };
	b2WorldId worldId = b2CreateWorld( &wd );

	b2BodyDef gd = b2DefaultBodyDef();
	gd.position = ( b2Vec2 ){ 0.0f, -10.0f };
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2Polygon groundBox = b2MakeBox( 50.0f, 10.0f );
	b2ShapeDef gsd = b2DefaultShapeDef();
	b2CreatePolygonShape( groundId, &gsd, &groundBox );

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.position = ( b2Vec2 ){ 0.0f, 4.0f };
	b2BodyId bodyId = b2CreateBody( worldId, &bd );
	b2Polygon box = b2MakeBox( 1.0f, 1.0f );
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.3f;
	b2CreatePolygonShape( bodyId, &sd, &box );
	if ( bodyOut )
		*bodyOut = bodyId;
	return worldId;
}

b2WorldId b2s_tilted_stacks( void )
{
	b2WorldDef wd = b2DefaultWorldDef();
	wd.gravity = ( b2Vec2 ){ 0.0f, -10.0f };
	wd.enableSleep = false;
	b2WorldId worldId = b2CreateWorld( &wd );

	b2BodyDef gd = b2DefaultBodyDef();
	gd.position = ( b2Vec2 ){ 0.0f, -1.0f };
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2Polygon ground = b2MakeBox( 1000.0f, 1.0f );
	b2ShapeDef gsd = b2DefaultShapeDef();
	b2CreatePolygonShape( groundId, &gsd, &ground );

	b2Polygon box = b2MakeRoundedBox( 0.45f, 0.45f, 0.05f );
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.3f;

	int columns = 10, rows = 10;
	float offset = 0.2f;
	float dx = 5.0f;
	float xroot = -0.5f * dx * ( columns - 1.0f );
	for ( int j = 0; j < columns; ++j )
	{
		float x = xroot + j * dx;
		for ( int i = 0; i < rows; ++i )
		{
			b2BodyDef bd = b2DefaultBodyDef();
			bd.type = b2_dynamicBody;
			bd.position = ( b2Vec2 ){ x + offset * i, 0.5f + 1.0f * i };
			b2BodyId bodyId = b2CreateBody( worldId, &bd );
			b2CreatePolygonShape( bodyId, &sd, &box );
		}
	}
	return worldId;
}

b2WorldId b2s_joint_grid( int n, float gravityY )
{
	b2WorldDef wd = b2s_world_def();
	wd.gravity = ( b2Vec2 ){ 0.0f, gravityY };
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) || n <= 0 )
		return worldId;

	/* column k holds the bodies k*n .. k*n + n - 1, top to bottom */
	b2BodyId* grid = (b2BodyId*)malloc( sizeof( b2BodyId ) * (size_t)n * (size_t)n );

	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.filter.categoryBits = 2;
	sd.filter.maskBits = ~2u;
	b2Circle circle = { { 0.0f, 0.0f }, 0.4f };

	b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
	b2BodyDef bd = b2DefaultBodyDef();
	bd.enableSleep = false;

	int at = 0;
	for ( int k = 0; k < n; ++k )
	{
		for ( int i = 0; i < n; ++i )
		{
			bool anchor = i == 0 && k >= n / 2 - 3 && k <= n / 2 + 3;
			bd.type = anchor ? b2_staticBody : b2_dynamicBody;
			bd.position = ( b2Vec2 ){ (float)k, -(float)i };
			b2BodyId body = b2CreateBody( worldId, &bd );
			b2CreateCircleShape( body, &sd, &circle );
			if ( i > 0 )
			{
				/* link to the body above */
				jd.bodyIdA = grid[at - 1];
				jd.bodyIdB = body;
				jd.localAnchorA = ( b2Vec2 ){ 0.0f, -0.5f };
				jd.localAnchorB = ( b2Vec2 ){ 0.0f, 0.5f };
				b2CreateRevoluteJoint( worldId, &jd );
			}
			if ( k > 0 )
			{
				/* link to the body on the left */
				jd.bodyIdA = grid[at - n];
				jd.bodyIdB = body;
				jd.localAnchorA = ( b2Vec2 ){ 0.5f, 0.0f };
				jd.localAnchorB = ( b2Vec2 ){ -0.5f, 0.0f };
				b2CreateRevoluteJoint( worldId, &jd );
			}
			grid[at++] = body;
		}
	}
	free( grid );
	return worldId;
}

b2WorldId b2s_many_pyramids( int rowCount, int columnCount, int baseCount )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;

	float extent = 0.5f;
	b2BodyDef gd = b2DefaultBodyDef();
	b2BodyId groundId = b2CreateBody( worldId, &gd );

	/* one ground segment under each row of pyramids, rows stacked groundDeltaY apart */
	float groundDeltaY = 2.0f * extent * ( baseCount + 1.0f );
	float groundWidth = 2.0f * extent * columnCount * ( baseCount + 1.0f );
	b2ShapeDef gsd = b2DefaultShapeDef();
	float groundY = 0.0f;
	for ( int i = 0; i < rowCount; ++i )
	{
		b2Segment segment = { { -0.5f * 2.0f * groundWidth, groundY }, { 0.5f * 2.0f * groundWidth, groundY } };
		b2CreateSegmentShape( groundId, &gsd, &segment );
		groundY += groundDeltaY;
	}

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2ShapeDef sd = b2DefaultShapeDef();
	b2Polygon box = b2MakeSquare( extent );
	float baseWidth = 2.0f * extent * baseCount;
	float baseY = 0.0f;
	for ( int r = 0; r < rowCount; ++r )
	{
		for ( int c = 0; c < columnCount; ++c )
		{
			float centerX = -0.5f * groundWidth + c * ( baseWidth + 2.0f * extent ) + extent;
			for ( int i = 0; i < baseCount; ++i )
			{
				float y = ( 2.0f * i + 1.0f ) * extent + baseY;
				for ( int j = i; j < baseCount; ++j )
				{
					float x = ( i + 1.0f ) * extent + 2.0f * ( j - i ) * extent + centerX - 0.5f;
					bd.position = ( b2Vec2 ){ x, y };
					b2BodyId bodyId = b2CreateBody( worldId, &bd );
					b2CreatePolygonShape( bodyId, &sd, &box );
				}
			}
		}
		baseY += groundDeltaY;
	}
	return worldId;
}

b2WorldId b2s_shape_pile( int count, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;

	/* static funnel: a floor segment, two sloped segments, a static capsule bar and a
	 * static box ledge */
	b2BodyDef gd = b2DefaultBodyDef();
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2ShapeDef gsd = b2DefaultShapeDef();
	b2Segment floorSeg = { { -12.0f, 0.0f }, { 12.0f, 0.0f } };
	b2CreateSegmentShape( groundId, &gsd, &floorSeg );
	b2Segment left = { { -12.0f, 0.0f }, { -16.0f, 12.0f } };
	b2CreateSegmentShape( groundId, &gsd, &left );
	b2Segment right = { { 12.0f, 0.0f }, { 16.0f, 12.0f } };
	b2CreateSegmentShape( groundId, &gsd, &right );
	b2Capsule bar = { { -4.0f, 3.0f }, { -1.0f, 2.0f }, 0.25f };
	b2CreateCapsuleShape( groundId, &gsd, &bar );
	b2Polygon ledge = b2MakeOffsetBox( 1.5f, 0.25f, ( b2Vec2 ){ 4.0f, 2.5f }, 0.0f );
	b2CreatePolygonShape( groundId, &gsd, &ledge );

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.6f;

	/* seeded jittered grid of 1 m cells above the funnel: 20 columns, rows upward;
	 * five shape kinds in turn */
	b2sRandom rng;
	b2s_seed( &rng, seed );
	b2Capsule capsule = { { -0.25f, 0.0f }, { 0.25f, 0.0f }, 0.3f };
	b2Capsule upright = { { 0.0f, -0.2f }, { 0.0f, 0.2f }, 0.3f };
	b2Polygon box = b2MakeBox( 0.35f, 0.3f );
	b2Polygon rounded = b2MakeRoundedBox( 0.25f, 0.2f, 0.1f );
	b2Circle circle = { { 0.0f, 0.0f }, 0.35f };
	for ( int k = 0; k < count; ++k )
	{
		int col = k % 20;
		int row = k / 20;
		float x = -9.5f + 1.0f * col + b2s_uniform( &rng, -0.05f, 0.05f );
		float y = 4.5f + 1.05f * row + b2s_uniform( &rng, -0.05f, 0.05f );
		bd.position = ( b2Vec2 ){ x, y };
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
		switch ( k % 5 )
		{
			case 0:
				b2CreateCapsuleShape( bodyId, &sd, &capsule );
				break;
			case 1:
				b2CreatePolygonShape( bodyId, &sd, &box );
				break;
			case 2:
				b2CreateCircleShape( bodyId, &sd, &circle );
				break;
			case 3:
				b2CreatePolygonShape( bodyId, &sd, &rounded );
				break;
			default:
				b2CreateCapsuleShape( bodyId, &sd, &upright );
				break;
		}
	}
	return worldId;
}

/* Point on the unit circle at parameter t in [-1, 1] (quarter turn per unit), by the
 * rational parametrisation ((1 - t^2), 2t) / (1 + t^2): float arithmetic only. */
static b2Vec2 b2s_circle_point( float t )
{
	float d = 1.0f + t * t;
	return ( b2Vec2 ){ ( 1.0f - t * t ) / d, 2.0f * t / d };
}

b2WorldId b2s_joint_hub( int spokes, int chains, int flags, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;
	b2s_ground( worldId, 0.6f );

	b2BodyDef anchorDef = b2DefaultBodyDef();
	b2BodyId anchorId = b2CreateBody( worldId, &anchorDef );

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.enableSleep = false;
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.6f;

	b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
	bool limits = ( flags & 1 ) != 0;
	bool springs = ( flags & 2 ) != 0;
	bool motor = ( flags & 4 ) != 0;

	/* hub: a circle of radius 1 at (0, 8) pinned to the static anchor */
	b2Vec2 hubCenter = { 0.0f, 8.0f };
	bd.position = hubCenter;
	b2BodyId hubId = b2CreateBody( worldId, &bd );
	b2Circle hubCircle = { { 0.0f, 0.0f }, 1.0f };
	b2CreateCircleShape( hubId, &sd, &hubCircle );
	jd.bodyIdA = anchorId;
	jd.bodyIdB = hubId;
	jd.localAnchorA = hubCenter;
	jd.localAnchorB = ( b2Vec2 ){ 0.0f, 0.0f };
	jd.enableMotor = motor;
	jd.motorSpeed = 1.0f;
	jd.maxMotorTorque = 2000.0f;
	b2CreateRevoluteJoint( worldId, &jd );

	/* spokes: boxes on a ring of radius 2.5 around the hub, each pinned to the hub at its
	 * own centre and to the next spoke; the hub's joints beyond the graph's colours go to
	 * the overflow set */
	b2Polygon spokeBox = b2MakeBox( 0.3f, 0.3f );
	b2BodyId first = b2_nullBodyId, prev = b2_nullBodyId;
	b2Vec2 prevPos = { 0.0f, 0.0f }, firstPos = { 0.0f, 0.0f };
	for ( int k = 0; k < spokes; ++k )
	{
		/* four quarter arcs of spokes / 4 points each */
		int quarter = ( 4 * k ) / ( spokes > 0 ? spokes : 1 );
		float t = -1.0f + 2.0f * ( (float)( 4 * k - quarter * spokes ) + 0.5f ) / (float)spokes;
		b2Vec2 u = b2s_circle_point( t );
		for ( int q = 0; q < quarter; ++q )
			u = ( b2Vec2 ){ -u.y, u.x };
		b2Vec2 offset = { 2.5f * u.x, 2.5f * u.y };
		b2Vec2 pos = { hubCenter.x + offset.x, hubCenter.y + offset.y };
		bd.position = pos;
		b2BodyId spokeId = b2CreateBody( worldId, &bd );
		b2CreatePolygonShape( spokeId, &sd, &spokeBox );

		jd = b2DefaultRevoluteJointDef();
		jd.bodyIdA = hubId;
		jd.bodyIdB = spokeId;
		jd.localAnchorA = offset;
		jd.localAnchorB = ( b2Vec2 ){ 0.0f, 0.0f };
		jd.enableLimit = limits;
		jd.lowerAngle = -0.2f * b2_pi;
		jd.upperAngle = 0.1f * b2_pi;
		jd.enableSpring = springs;
		jd.hertz = 1.5f;
		jd.dampingRatio = 0.4f;
		jd.enableMotor = motor && ( k % 3 ) == 0;
		jd.motorSpeed = ( k & 1 ) ? 0.5f : -0.5f;
		jd.maxMotorTorque = 5.0f;
		b2CreateRevoluteJoint( worldId, &jd );

		if ( k > 0 )
		{
			jd = b2DefaultRevoluteJointDef();
			jd.bodyIdA = prev;
			jd.bodyIdB = spokeId;
			b2Vec2 mid = { 0.5f * ( prevPos.x + pos.x ), 0.5f * ( prevPos.y + pos.y ) };
			jd.localAnchorA = ( b2Vec2 ){ mid.x - prevPos.x, mid.y - prevPos.y };
			jd.localAnchorB = ( b2Vec2 ){ mid.x - pos.x, mid.y - pos.y };
			b2CreateRevoluteJoint( worldId, &jd );
		}
		else
		{
			first = spokeId;
			firstPos = pos;
		}
		prev = spokeId;
		prevPos = pos;
	}
	if ( spokes > 2 )
	{
		jd = b2DefaultRevoluteJointDef();
		jd.bodyIdA = prev;
		jd.bodyIdB = first;
		b2Vec2 mid = { 0.5f * ( prevPos.x + firstPos.x ), 0.5f * ( prevPos.y + firstPos.y ) };
		jd.localAnchorA = ( b2Vec2 ){ mid.x - prevPos.x, mid.y - prevPos.y };
		jd.localAnchorB = ( b2Vec2 ){ mid.x - firstPos.x, mid.y - firstPos.y };
		b2CreateRevoluteJoint( worldId, &jd );
	}

	/* chains: capsule links of length 0.5 hanging from static pins on a line at y = 14,
	 * laid out along a 45 degree diagonal so they swing down; adjacent links are jointed
	 * and do not collide */
	b2sRandom rng;
	b2s_seed( &rng, seed );
	b2Capsule link = { { -0.25f, 0.0f }, { 0.25f, 0.0f }, 0.2f };
	const int links = 6;
	for ( int c = 0; c < chains; ++c )
	{
		b2Vec2 pin = { -12.0f + 4.0f * c, 14.0f };
		b2BodyId above = anchorId;
		b2Vec2 aboveAnchor = pin;
		for ( int i = 0; i < links; ++i )
		{
			/* link i spans pin + d * (i, i+1) along d = (0.3536, -0.3536) */
			float s = 0.35355339f;
			b2Vec2 center = { pin.x + s * ( i + 0.5f ), pin.y - s * ( i + 0.5f ) };
			bd.position = center;
			bd.rotation = ( b2Rot ){ 0.70710678f, -0.70710678f };
			bd.angularVelocity = b2s_uniform( &rng, -0.5f, 0.5f );
			b2BodyId linkId = b2CreateBody( worldId, &bd );
			b2CreateCapsuleShape( linkId, &sd, &link );

			jd = b2DefaultRevoluteJointDef();
			jd.bodyIdA = above;
			jd.bodyIdB = linkId;
			jd.localAnchorA = aboveAnchor;
			jd.localAnchorB = ( b2Vec2 ){ -0.25f, 0.0f };
			jd.referenceAngle = i == 0 ? -0.25f * b2_pi : 0.0f;
			jd.enableLimit = limits;
			jd.lowerAngle = -0.3f * b2_pi;
			jd.upperAngle = 0.3f * b2_pi;
			jd.enableSpring = springs && ( i & 1 ) == 0;
			jd.hertz = 3.0f;
			jd.dampingRatio = 0.7f;
			b2CreateRevoluteJoint( worldId, &jd );

			above = linkId;
			aboveAnchor = ( b2Vec2 ){ 0.25f, 0.0f };
		}
	}
	bd.rotation = b2Rot_identity;
	bd.angularVelocity = 0.0f;

	/* a few boxes dropped onto the spokes and the chains */
	b2Polygon box = b2MakeBox( 0.4f, 0.4f );
	for ( int k = 0; k < 12; ++k )
	{
		bd.position = ( b2Vec2 ){ -6.0f + 1.1f * k + b2s_uniform( &rng, -0.1f, 0.1f ), 12.0f + 0.5f * ( k & 1 ) };
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
		b2CreatePolygonShape( bodyId, &sd, &box );
	}
	return worldId;
}

b2WorldId b2s_fast_shots( int count, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;

	/* static: a ground segment and a 0.1 m thick wall at x = 20 */
	b2BodyDef gd = b2DefaultBodyDef();
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2ShapeDef gsd = b2DefaultShapeDef();
	b2Segment floorSeg = { { -10.0f, 0.0f }, { 40.0f, 0.0f } };
	b2CreateSegmentShape( groundId, &gsd, &floorSeg );
	b2Polygon wall = b2MakeOffsetBox( 0.05f, 10.0f, ( b2Vec2 ){ 20.0f, 10.0f }, 0.0f );
	b2CreatePolygonShape( groundId, &gsd, &wall );

	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.6f;
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;

	/* a column of boxes standing in front of the wall: bullets sweep against them */
	b2Polygon block = b2MakeBox( 0.4f, 0.4f );
	for ( int i = 0; i < 10; ++i )
	{
		bd.position = ( b2Vec2 ){ 15.0f, 0.4f + 0.8f * i };
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
		b2CreatePolygonShape( bodyId, &sd, &block );
	}

	/* projectiles fired at the wall at 60 to 120 m/s: circles, boxes and capsules in
	 * turn; every fourth is a bullet */
	b2sRandom rng;
	b2s_seed( &rng, seed );
	b2Circle circle = { { 0.0f, 0.0f }, 0.1f };
	b2Polygon box = b2MakeBox( 0.1f, 0.1f );
	b2Capsule capsule = { { -0.1f, 0.0f }, { 0.1f, 0.0f }, 0.08f };
	for ( int k = 0; k < count; ++k )
	{
		float px = b2s_uniform( &rng, 0.0f, 5.0f );
		float py = b2s_uniform( &rng, 1.0f, 15.0f );
		float vx = b2s_uniform( &rng, 60.0f, 120.0f );
		float vy = b2s_uniform( &rng, -5.0f, 5.0f );
		bd.position = ( b2Vec2 ){ px, py };
		bd.linearVelocity = ( b2Vec2 ){ vx, vy };
		bd.angularVelocity = b2s_uniform( &rng, -10.0f, 10.0f );
		bd.isBullet = ( k & 3 ) == 3;
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
		switch ( k % 3 )
		{
			case 0:
				b2CreateCircleShape( bodyId, &sd, &circle );
				break;
			case 1:
				b2CreatePolygonShape( bodyId, &sd, &box );
				break;
			default:
				b2CreateCapsuleShape( bodyId, &sd, &capsule );
				break;
		}
	}
	return worldId;
}

/* Rotation with the direction of (x, y): sqrtf and division only. */
static b2Rot b2s_unit( float x, float y )
{
	float len = sqrtf( x * x + y * y );
	return ( b2Rot ){ x / len, y / len };
}

b2WorldId b2s_joint_chains( int chains, int links, int flags, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;

	b2BodyDef anchorDef = b2DefaultBodyDef();
	b2BodyId anchorId = b2CreateBody( worldId, &anchorDef );

	/* links never touch: one category that its own mask excludes */
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.filter.categoryBits = 4;
	sd.filter.maskBits = ~4u;
	b2Capsule link = { { -0.25f, 0.0f }, { 0.25f, 0.0f }, 0.1f };

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.enableSleep = false;
	bd.angularDamping = 0.1f;

	b2sRandom rng;
	b2s_seed( &rng, seed );
	for ( int c = 0; c < chains; ++c )
	{
		b2Vec2 pin = { 3.0f * c, 0.0f };
		/* chains start along a line tilted by a seeded slope below the horizontal */
		float slope = b2s_uniform( &rng, 0.2f, 1.0f );
		b2Rot rot = b2s_unit( 1.0f, -slope );
		b2BodyId above = anchorId;
		b2Vec2 aboveAnchor = pin;
		for ( int i = 0; i < links; ++i )
		{
			b2Vec2 center = { pin.x + rot.c * 0.5f * ( i + 0.5f ), pin.y + rot.s * 0.5f * ( i + 0.5f ) };
			bd.position = center;
			bd.rotation = rot;
			b2BodyId linkId = b2CreateBody( worldId, &bd );
			b2CreateCapsuleShape( linkId, &sd, &link );

			b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
			jd.bodyIdA = above;
			jd.bodyIdB = linkId;
			jd.localAnchorA = aboveAnchor;
			jd.localAnchorB = ( b2Vec2 ){ -0.25f, 0.0f };
			jd.enableLimit = ( flags & 1 ) != 0;
			jd.lowerAngle = -0.3f * b2_pi;
			jd.upperAngle = 0.15f * b2_pi;
			jd.enableSpring = ( flags & 2 ) != 0;
			jd.hertz = 2.0f;
			jd.dampingRatio = 0.5f;
			jd.enableMotor = ( flags & 4 ) != 0 && ( i % 3 ) == 1;
			jd.motorSpeed = ( c & 1 ) ? 0.5f : -0.5f;
			jd.maxMotorTorque = 2.0f;
			b2CreateRevoluteJoint( worldId, &jd );

			above = linkId;
			aboveAnchor = ( b2Vec2 ){ 0.25f, 0.0f };
		}
	}
	return worldId;
}

/* ids of the destruction scene, per process (one such scene at a time) */
static struct
{
	b2BodyId pyramid[55];
	b2BodyId hub;
	b2BodyId spokes[14];
	b2JointId spokeJoints[14];
	b2BodyId pairs[6];
	b2ShapeId pairShapes[6][2];
	b2ShapeId ledge;
} s_destruction;

b2WorldId b2s_destruction( void )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;
	memset( &s_destruction, 0, sizeof( s_destruction ) );

	b2BodyDef gd = b2DefaultBodyDef();
	gd.position = ( b2Vec2 ){ 0.0f, -0.5f };
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2ShapeDef gsd = b2DefaultShapeDef();
	b2Polygon groundBox = b2MakeBox( 40.0f, 0.5f );
	b2CreatePolygonShape( groundId, &gsd, &groundBox );
	b2Polygon ledge = b2MakeOffsetBox( 2.0f, 0.25f, ( b2Vec2 ){ 12.0f, 4.0f }, 0.0f );
	s_destruction.ledge = b2CreatePolygonShape( groundId, &gsd, &ledge );

	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.6f;

	/* a 10-row pyramid of unit boxes left of the origin */
	b2Polygon box = b2MakeSquare( 0.5f );
	int n = 0;
	for ( int i = 0; i < 10; ++i )
	{
		for ( int j = i; j < 10; ++j )
		{
			bd.position = ( b2Vec2 ){ -15.0f + ( i + 1.0f ) * 0.5f + ( j - i ) * 1.0f, ( 2.0f * i + 1.0f ) * 0.5f };
			s_destruction.pyramid[n] = b2CreateBody( worldId, &bd );
			b2CreatePolygonShape( s_destruction.pyramid[n], &sd, &box );
			n += 1;
		}
	}

	/* a hub pinned to a shapeless static anchor with 14 spokes pinned to it (the joints
	 * beyond the graph's colours go to the overflow set) */
	b2BodyDef ad = b2DefaultBodyDef();
	b2BodyId anchorId = b2CreateBody( worldId, &ad );
	bd.position = ( b2Vec2 ){ 0.0f, 6.0f };
	s_destruction.hub = b2CreateBody( worldId, &bd );
	b2Circle hubCircle = { { 0.0f, 0.0f }, 0.8f };
	b2CreateCircleShape( s_destruction.hub, &sd, &hubCircle );
	b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
	jd.bodyIdA = anchorId;
	jd.bodyIdB = s_destruction.hub;
	jd.localAnchorA = ( b2Vec2 ){ 0.0f, 6.0f };
	b2CreateRevoluteJoint( worldId, &jd );
	b2Polygon spokeBox = b2MakeBox( 0.25f, 0.25f );
	for ( int k = 0; k < 14; ++k )
	{
		b2Vec2 u = b2s_circle_point( -1.0f + 2.0f * ( k + 0.5f ) / 14.0f );
		b2Vec2 offset = { 2.0f * u.x, 2.0f * u.y };
		bd.position = ( b2Vec2 ){ offset.x, 6.0f + offset.y };
		s_destruction.spokes[k] = b2CreateBody( worldId, &bd );
		b2CreatePolygonShape( s_destruction.spokes[k], &sd, &spokeBox );
		jd = b2DefaultRevoluteJointDef();
		jd.bodyIdA = s_destruction.hub;
		jd.bodyIdB = s_destruction.spokes[k];
		jd.localAnchorA = offset;
		s_destruction.spokeJoints[k] = b2CreateRevoluteJoint( worldId, &jd );
	}

	/* bodies of two shapes each (a box and a capsule) dropped onto the ledge */
	b2Capsule cap = { { -0.3f, 0.0f }, { 0.3f, 0.0f }, 0.2f };
	b2Polygon small = b2MakeOffsetBox( 0.2f, 0.2f, ( b2Vec2 ){ 0.0f, 0.4f }, 0.0f );
	for ( int k = 0; k < 6; ++k )
	{
		bd.position = ( b2Vec2 ){ 10.5f + 0.6f * k, 5.0f + 1.2f * k };
		s_destruction.pairs[k] = b2CreateBody( worldId, &bd );
		s_destruction.pairShapes[k][0] = b2CreateCapsuleShape( s_destruction.pairs[k], &sd, &cap );
		s_destruction.pairShapes[k][1] = b2CreatePolygonShape( s_destruction.pairs[k], &sd, &small );
	}
	return worldId;
}

void b2s_destruction_step( b2WorldId worldId, int step )
{
	if ( step == 20 )
	{
		/* bodies inside the pyramid: the awake order changes by swap-removal */
		int doomed[5] = { 3, 12, 27, 40, 54 };
		for ( int i = 0; i < 5; ++i )
			b2DestroyBody( s_destruction.pyramid[doomed[i]] );
	}
	else if ( step == 40 )
	{
		/* spoke joints, in the graph colours and in the overflow set */
		int doomed[4] = { 0, 5, 11, 13 };
		for ( int i = 0; i < 4; ++i )
			b2DestroyJoint( s_destruction.spokeJoints[doomed[i]] );
	}
	else if ( step == 60 )
	{
		/* one shape of each two-shape body: contacts go, masses are recomputed */
		for ( int k = 0; k < 6; ++k )
			b2DestroyShape( s_destruction.pairShapes[k][k & 1] );
	}
	else if ( step == 80 )
	{
		/* the hub with its remaining joints and contacts */
		b2DestroyBody( s_destruction.hub );
	}
	else if ( step == 100 )
	{
		/* new bodies take the freed ids */
		b2BodyDef bd = b2DefaultBodyDef();
		bd.type = b2_dynamicBody;
		b2ShapeDef sd = b2DefaultShapeDef();
		b2Polygon box = b2MakeSquare( 0.4f );
		for ( int k = 0; k < 8; ++k )
		{
			bd.position = ( b2Vec2 ){ -4.0f + 1.0f * k, 3.0f };
			b2BodyId id = b2CreateBody( worldId, &bd );
			b2CreatePolygonShape( id, &sd, &box );
		}
	}
	else if ( step == 120 )
	{
		/* a static shape under resting bodies */
		b2DestroyShape( s_destruction.ledge );
	}
}

b2WorldId b2s_empty_world( void )
{
	b2WorldDef wd = b2DefaultWorldDef();
	return b2CreateWorld( &wd );
}

b2BodyId b2s_add_body( b2WorldId worldId, int type )
{
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = (b2BodyType)type;
	return b2CreateBody( worldId, &bd );
}

b2BodyId b2s_add_square( b2WorldId worldId, float h )
{
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2BodyId bodyId = b2CreateBody( worldId, &bd );
	b2ShapeDef sd = b2DefaultShapeDef();
	b2Polygon square = b2MakeSquare( h );
	b2CreatePolygonShape( bodyId, &sd, &square );
	return bodyId;
}

b2WorldId b2s_event_scene( int count, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;

	/* ground with hit events; a static sensor band the bodies fall through */
	b2BodyDef gd = b2DefaultBodyDef();
	gd.position = ( b2Vec2 ){ 0.0f, -0.5f };
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2ShapeDef gsd = b2DefaultShapeDef();
	gsd.enableHitEvents = true;
	b2Polygon groundBox = b2MakeBox( 30.0f, 0.5f );
	b2CreatePolygonShape( groundId, &gsd, &groundBox );
	b2ShapeDef sensorDef = b2DefaultShapeDef();
	sensorDef.isSensor = true;
	b2Polygon band = b2MakeOffsetBox( 12.0f, 0.75f, ( b2Vec2 ){ 0.0f, 4.5f }, 0.0f );
	b2CreatePolygonShape( groundId, &sensorDef, &band );

	b2sRandom rng;
	b2s_seed( &rng, seed );
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2Polygon box = b2MakeBox( 0.3f, 0.3f );
	b2Circle circle = { { 0.0f, 0.0f }, 0.3f };
	b2Circle ring = { { 0.0f, 0.0f }, 0.8f };
	for ( int k = 0; k < count; ++k )
	{
		float jx = b2s_uniform( &rng, -0.1f, 0.1f );
		float jy = b2s_uniform( &rng, 0.0f, 1.0f );
		bd.position = ( b2Vec2 ){ -10.0f + 20.0f * ( k + 0.5f ) / count + jx, 6.0f + 2.5f * ( k % 3 ) + jy };
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
		b2ShapeDef sd = b2DefaultShapeDef();
		sd.density = 1.0f;
		sd.friction = 0.5f;
		sd.restitution = ( k % 4 ) == 0 ? 0.6f : 0.1f;
		sd.enableHitEvents = ( k & 1 ) == 0;
		sd.enableContactEvents = ( k % 5 ) != 4;
		if ( k % 2 == 0 )
			b2CreatePolygonShape( bodyId, &sd, &box );
		else
			b2CreateCircleShape( bodyId, &sd, &circle );
		if ( k % 7 == 3 )
		{
			/* a sensor ring carried by the body */
			b2ShapeDef ringDef = b2DefaultShapeDef();
			ringDef.isSensor = true;
			ringDef.density = 0.0f;
			b2CreateCircleShape( bodyId, &ringDef, &ring );
		}
	}
	return worldId;
}

/* One copy of the joint scene at x offset x0 on the shared static ground. */
static void b2s_zoo_copy( b2WorldId worldId, b2BodyId groundId, float x0, int flags, b2sRandom* rng )
{
	bool collide = ( flags & 1 ) != 0;
	b2ShapeDef sd = b2DefaultShapeDef();
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2BodyDef sb = b2DefaultBodyDef();

	/* distance rope: six circles from a static pin, alternating soft-with-limits, rigid,
	 * and motorised links */
	{
		sb.position = ( b2Vec2 ){ x0 - 15.0f, 12.0f };
		b2BodyId pin = b2CreateBody( worldId, &sb );
		b2Circle ball = { { 0.0f, 0.0f }, 0.25f };
		b2BodyId prev = pin;
		for ( int i = 0; i < 6; ++i )
		{
			bd.position = ( b2Vec2 ){ x0 - 15.0f + 1.0f * ( i + 1 ), 12.0f - 0.2f * ( i + 1 ) };
			b2BodyId link = b2CreateBody( worldId, &bd );
			b2CreateCircleShape( link, &sd, &ball );
			b2DistanceJointDef dj = b2DefaultDistanceJointDef();
			dj.bodyIdA = prev;
			dj.bodyIdB = link;
			dj.length = 1.0f;
			dj.collideConnected = collide;
			if ( i % 3 == 0 )
			{
				dj.enableSpring = true;
				dj.hertz = 3.0f;
				dj.dampingRatio = 0.4f;
				dj.enableLimit = true;
				dj.minLength = 0.8f;
				dj.maxLength = 1.25f;
			}
			else if ( i % 3 == 2 )
			{
				dj.enableSpring = true;
				dj.hertz = 2.0f;
				dj.dampingRatio = 0.2f;
				dj.enableMotor = true;
				dj.maxMotorForce = 20.0f;
				dj.motorSpeed = 0.5f;
			}
			b2CreateDistanceJoint( worldId, &dj );
			prev = link;
		}
	}

	/* revolute pendulum with spring, limits and motor */
	{
		sb.position = ( b2Vec2 ){ x0 - 3.0f, 8.0f };
		b2BodyId pin = b2CreateBody( worldId, &sb );
		bd.position = ( b2Vec2 ){ x0 - 1.5f, 8.0f };
		b2BodyId bob = b2CreateBody( worldId, &bd );
		b2Polygon box = b2MakeBox( 1.5f, 0.2f );
		b2CreatePolygonShape( bob, &sd, &box );
		b2RevoluteJointDef rj = b2DefaultRevoluteJointDef();
		rj.bodyIdA = pin;
		rj.bodyIdB = bob;
		rj.localAnchorB = ( b2Vec2 ){ -1.5f, 0.0f };
		rj.enableSpring = true;
		rj.hertz = 1.0f;
		rj.dampingRatio = 0.3f;
		rj.enableLimit = true;
		rj.lowerAngle = -0.4f * b2_pi;
		rj.upperAngle = 0.25f * b2_pi;
		rj.enableMotor = true;
		rj.maxMotorTorque = 10.0f;
		rj.motorSpeed = 0.3f;
		b2CreateRevoluteJoint( worldId, &rj );
	}

	/* prismatic elevators: a motorised platform with limits, a spring platform on a tilted
	 * axis, each with a box on top */
	for ( int k = 0; k < 2; ++k )
	{
		float x = x0 + 1.0f + 3.0f * k;
		bd.position = ( b2Vec2 ){ x, 1.0f };
		b2BodyId plat = b2CreateBody( worldId, &bd );
		b2Polygon slab = b2MakeBox( 1.0f, 0.15f );
		b2CreatePolygonShape( plat, &sd, &slab );
		b2PrismaticJointDef pj = b2DefaultPrismaticJointDef();
		pj.bodyIdA = groundId;
		pj.bodyIdB = plat;
		pj.localAnchorA = ( b2Vec2 ){ x, 1.0f };
		pj.localAxisA = k == 0 ? ( b2Vec2 ){ 0.0f, 1.0f } : ( b2Vec2 ){ 0.3f, 1.0f };
		pj.collideConnected = collide;
		if ( k == 0 )
		{
			pj.enableLimit = true;
			pj.lowerTranslation = -0.5f;
			pj.upperTranslation = 3.0f;
			pj.enableMotor = true;
			pj.maxMotorForce = 300.0f;
			pj.motorSpeed = 1.0f;
		}
		else
		{
			pj.enableSpring = true;
			pj.hertz = 2.0f;
			pj.dampingRatio = 0.5f;
			pj.enableLimit = true;
			pj.lowerTranslation = -0.75f;
			pj.upperTranslation = 2.0f;
		}
		b2CreatePrismaticJoint( worldId, &pj );
		bd.position = ( b2Vec2 ){ x + 0.2f, 1.6f };
		b2BodyId cargo = b2CreateBody( worldId, &bd );
		b2Polygon cbox = b2MakeBox( 0.4f, 0.4f );
		b2CreatePolygonShape( cargo, &sd, &cbox );
	}

	/* wheel car: chassis, two wheels on sprung axles with travel limits, rear motor */
	{
		float cx = x0 + 8.0f;
		bd.position = ( b2Vec2 ){ cx, 1.2f };
		b2BodyId chassis = b2CreateBody( worldId, &bd );
		b2Polygon body = b2MakeBox( 1.2f, 0.25f );
		b2CreatePolygonShape( chassis, &sd, &body );
		b2Circle tire = { { 0.0f, 0.0f }, 0.4f };
		b2ShapeDef wsd = b2DefaultShapeDef();
		wsd.friction = 1.5f;
		for ( int k = 0; k < 2; ++k )
		{
			float wx = cx + ( k == 0 ? -0.9f : 0.9f );
			bd.position = ( b2Vec2 ){ wx, 0.5f };
			b2BodyId wheel = b2CreateBody( worldId, &bd );
			b2CreateCircleShape( wheel, &wsd, &tire );
			b2WheelJointDef wj = b2DefaultWheelJointDef();
			wj.bodyIdA = chassis;
			wj.bodyIdB = wheel;
			wj.localAnchorA = ( b2Vec2 ){ k == 0 ? -0.9f : 0.9f, -0.7f };
			wj.hertz = 5.0f;
			wj.dampingRatio = 0.7f;
			wj.enableLimit = true;
			wj.lowerTranslation = -0.25f;
			wj.upperTranslation = 0.25f;
			wj.enableMotor = k == 0;
			wj.maxMotorTorque = 15.0f;
			wj.motorSpeed = -3.0f;
			b2CreateWheelJoint( worldId, &wj );
		}
	}

	/* weld cantilever: five planks from a static wall, rigid and soft welds in turn */
	{
		sb.position = ( b2Vec2 ){ x0 + 12.0f, 6.0f };
		b2BodyId wall = b2CreateBody( worldId, &sb );
		b2Polygon post = b2MakeBox( 0.25f, 0.5f );
		b2CreatePolygonShape( wall, &sd, &post );
		b2Polygon plank = b2MakeBox( 0.5f, 0.125f );
		b2BodyId prev = wall;
		float prevHalf = 0.25f;
		for ( int i = 0; i < 5; ++i )
		{
			bd.position = ( b2Vec2 ){ x0 + 12.0f + 0.25f + 0.5f + 1.0f * i, 6.0f };
			b2BodyId p = b2CreateBody( worldId, &bd );
			b2CreatePolygonShape( p, &sd, &plank );
			b2WeldJointDef wj = b2DefaultWeldJointDef();
			wj.bodyIdA = prev;
			wj.bodyIdB = p;
			wj.localAnchorA = ( b2Vec2 ){ prevHalf, 0.0f };
			wj.localAnchorB = ( b2Vec2 ){ -0.5f, 0.0f };
			wj.referenceAngle = i == 2 ? 0.05f : 0.0f;
			if ( i & 1 )
			{
				wj.linearHertz = 6.0f;
				wj.linearDampingRatio = 0.7f;
				wj.angularHertz = 3.0f;
				wj.angularDampingRatio = 0.5f;
			}
			b2CreateWeldJoint( worldId, &wj );
			prev = p;
			prevHalf = 0.5f;
		}
	}

	/* motor joint: a box held at a moving offset from the ground with limited force */
	{
		bd.position = ( b2Vec2 ){ x0 + 19.0f, 2.0f };
		b2BodyId b = b2CreateBody( worldId, &bd );
		b2Polygon box = b2MakeBox( 0.5f, 0.5f );
		b2CreatePolygonShape( b, &sd, &box );
		b2MotorJointDef mj = b2DefaultMotorJointDef();
		mj.bodyIdA = groundId;
		mj.bodyIdB = b;
		mj.linearOffset = ( b2Vec2 ){ x0 + 19.0f, 3.0f };
		mj.angularOffset = 0.5f;
		mj.maxForce = 200.0f;
		mj.maxTorque = 40.0f;
		mj.correctionFactor = 0.3f;
		mj.collideConnected = true;
		b2CreateMotorJoint( worldId, &mj );
	}

	/* mouse joint: a circle pulled toward a target above and to the side */
	{
		bd.position = ( b2Vec2 ){ x0 - 8.0f, 0.6f };
		b2BodyId b = b2CreateBody( worldId, &bd );
		b2Circle c = { { 0.0f, 0.0f }, 0.5f };
		b2CreateCircleShape( b, &sd, &c );
		b2MouseJointDef mj = b2DefaultMouseJointDef();
		mj.bodyIdA = groundId;
		mj.bodyIdB = b;
		mj.target = ( b2Vec2 ){ x0 - 6.0f, 5.0f };
		mj.hertz = 3.0f;
		mj.dampingRatio = 0.7f;
		mj.maxForce = 60.0f;
		b2CreateMouseJoint( worldId, &mj );
	}

	/* spider: a hub box with fourteen legs of every joint type, so that the hub's
	 * constraints overflow the eleven graph colours */
	{
		float hx = x0 - 11.0f;
		bd.position = ( b2Vec2 ){ hx, 4.0f };
		b2BodyId hub = b2CreateBody( worldId, &bd );
		b2Polygon hubBox = b2MakeBox( 0.6f, 0.6f );
		b2CreatePolygonShape( hub, &sd, &hubBox );
		b2Polygon leg = b2MakeBox( 0.2f, 0.1f );
		for ( int k = 0; k < 14; ++k )
		{
			b2Vec2 u = b2s_circle_point( -1.0f + 2.0f * ( k + 0.5f ) / 14.0f );
			b2Vec2 at = { hx + 1.6f * u.x, 4.0f + 1.6f * u.y };
			bd.position = at;
			b2BodyId l = b2CreateBody( worldId, &bd );
			b2CreatePolygonShape( l, &sd, &leg );
			b2Vec2 anchor = { 0.6f * u.x, 0.6f * u.y };
			switch ( k % 7 )
			{
				case 0:
				{
					b2DistanceJointDef j = b2DefaultDistanceJointDef();
					j.bodyIdA = hub;
					j.bodyIdB = l;
					j.localAnchorA = anchor;
					j.length = 1.0f;
					j.enableSpring = true;
					j.hertz = 4.0f;
					j.dampingRatio = 0.5f;
					b2CreateDistanceJoint( worldId, &j );
					break;
				}
				case 1:
				{
					b2RevoluteJointDef j = b2DefaultRevoluteJointDef();
					j.bodyIdA = hub;
					j.bodyIdB = l;
					j.localAnchorA = anchor;
					j.localAnchorB = ( b2Vec2 ){ -1.0f * u.x, -1.0f * u.y };
					j.enableLimit = true;
					j.lowerAngle = -0.25f;
					j.upperAngle = 0.25f;
					b2CreateRevoluteJoint( worldId, &j );
					break;
				}
				case 2:
				{
					b2PrismaticJointDef j = b2DefaultPrismaticJointDef();
					j.bodyIdA = hub;
					j.bodyIdB = l;
					j.localAnchorA = anchor;
					j.localAnchorB = ( b2Vec2 ){ -1.0f * u.x, -1.0f * u.y };
					j.localAxisA = u;
					j.enableSpring = true;
					j.hertz = 3.0f;
					j.dampingRatio = 0.6f;
					j.enableLimit = true;
					j.lowerTranslation = -0.3f;
					j.upperTranslation = 0.3f;
					b2CreatePrismaticJoint( worldId, &j );
					break;
				}
				case 3:
				{
					b2WheelJointDef j = b2DefaultWheelJointDef();
					j.bodyIdA = hub;
					j.bodyIdB = l;
					j.localAnchorA = anchor;
					j.localAnchorB = ( b2Vec2 ){ -1.0f * u.x, -1.0f * u.y };
					j.localAxisA = u;
					j.enableMotor = true;
					j.maxMotorTorque = 2.0f;
					j.motorSpeed = 1.0f;
					b2CreateWheelJoint( worldId, &j );
					break;
				}
				case 4:
				{
					b2WeldJointDef j = b2DefaultWeldJointDef();
					j.bodyIdA = hub;
					j.bodyIdB = l;
					j.localAnchorA = anchor;
					j.localAnchorB = ( b2Vec2 ){ -1.0f * u.x, -1.0f * u.y };
					j.linearHertz = 8.0f;
					j.linearDampingRatio = 1.0f;
					j.angularHertz = 4.0f;
					j.angularDampingRatio = 1.0f;
					b2CreateWeldJoint( worldId, &j );
					break;
				}
				case 5:
				{
					b2MotorJointDef j = b2DefaultMotorJointDef();
					j.bodyIdA = hub;
					j.bodyIdB = l;
					j.linearOffset = ( b2Vec2 ){ 1.6f * u.x, 1.6f * u.y };
					j.maxForce = 50.0f;
					j.maxTorque = 5.0f;
					b2CreateMotorJoint( worldId, &j );
					break;
				}
				default:
				{
					b2MouseJointDef j = b2DefaultMouseJointDef();
					j.bodyIdA = hub;
					j.bodyIdB = l;
					j.target = ( b2Vec2 ){ at.x + 0.5f * u.x, at.y + 0.5f * u.y };
					j.hertz = 5.0f;
					j.dampingRatio = 0.8f;
					j.maxForce = 30.0f;
					b2CreateMouseJoint( worldId, &j );
					break;
				}
			}
		}
	}

	/* debris: seeded boxes and circles dropped over the mechanisms */
	for ( int k = 0; k < 12; ++k )
	{
		float px = x0 + b2s_uniform( rng, -16.0f, 20.0f );
		float py = b2s_uniform( rng, 8.0f, 14.0f );
		bd.position = ( b2Vec2 ){ px, py };
		b2BodyId d = b2CreateBody( worldId, &bd );
		if ( k & 1 )
		{
			b2Circle c = { { 0.0f, 0.0f }, b2s_uniform( rng, 0.15f, 0.35f ) };
			b2CreateCircleShape( d, &sd, &c );
		}
		else
		{
			float hx = b2s_uniform( rng, 0.15f, 0.4f );
			float hy = b2s_uniform( rng, 0.15f, 0.4f );
			b2Polygon p = b2MakeBox( hx, hy );
			b2CreatePolygonShape( d, &sd, &p );
		}
	}
}

b2WorldId b2s_joint_zoo( int copies, int flags, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;
	b2BodyDef gd = b2DefaultBodyDef();
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2ShapeDef gsd = b2DefaultShapeDef();
	float half = 20.0f * copies + 10.0f;
	b2Polygon groundBox = b2MakeOffsetBox( half, 0.5f, ( b2Vec2 ){ 40.0f * 0.5f * ( copies - 1 ), -0.5f }, 0.0f );
	b2CreatePolygonShape( groundId, &gsd, &groundBox );

	b2sRandom rng;
	b2s_seed( &rng, seed );
	for ( int i = 0; i < copies; ++i )
		b2s_zoo_copy( worldId, groundId, 40.0f * i, flags, &rng );
	return worldId;
}

/* Records a float into the script's output. */
static void b2s_put( float* out, int capacity, int* n, float v )
{
	if ( *n < capacity )
		out[*n] = v;
	*n += 1;
}

static void b2s_put_vec( float* out, int capacity, int* n, b2Vec2 v )
{
	b2s_put( out, capacity, n, v.x );
	b2s_put( out, capacity, n, v.y );
}

/* Reads back every joint's configuration, its reaction force and torque, and the
 * type-specific queries. */
static void b2s_joint_readout( b2JointId* j, float* out, int capacity, int* n )
{
	for ( int k = 0; k < 7; ++k )
	{
		b2s_put( out, capacity, n, (float)b2Joint_GetType( j[k] ) );
		b2s_put_vec( out, capacity, n, b2Joint_GetLocalAnchorA( j[k] ) );
		b2s_put_vec( out, capacity, n, b2Joint_GetLocalAnchorB( j[k] ) );
		b2s_put( out, capacity, n, b2Joint_GetCollideConnected( j[k] ) ? 1.0f : 0.0f );
		b2s_put_vec( out, capacity, n, b2Joint_GetConstraintForce( j[k] ) );
		b2s_put( out, capacity, n, b2Joint_GetConstraintTorque( j[k] ) );
	}
	b2JointId d = j[0];
	b2s_put( out, capacity, n, b2DistanceJoint_GetLength( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_IsSpringEnabled( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetHertz( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetDampingRatio( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_IsLimitEnabled( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetMinLength( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetMaxLength( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetCurrentLength( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_IsMotorEnabled( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetMotorSpeed( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetMaxMotorForce( d ) );
	b2s_put( out, capacity, n, b2DistanceJoint_GetMotorForce( d ) );
	b2JointId m = j[1];
	b2s_put_vec( out, capacity, n, b2MotorJoint_GetLinearOffset( m ) );
	b2s_put( out, capacity, n, b2MotorJoint_GetAngularOffset( m ) );
	b2s_put( out, capacity, n, b2MotorJoint_GetMaxForce( m ) );
	b2s_put( out, capacity, n, b2MotorJoint_GetMaxTorque( m ) );
	b2s_put( out, capacity, n, b2MotorJoint_GetCorrectionFactor( m ) );
	b2JointId o = j[2];
	b2s_put_vec( out, capacity, n, b2MouseJoint_GetTarget( o ) );
	b2s_put( out, capacity, n, b2MouseJoint_GetSpringHertz( o ) );
	b2s_put( out, capacity, n, b2MouseJoint_GetSpringDampingRatio( o ) );
	b2s_put( out, capacity, n, b2MouseJoint_GetMaxForce( o ) );
	b2JointId p = j[3];
	b2s_put( out, capacity, n, b2PrismaticJoint_IsSpringEnabled( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_GetSpringHertz( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_GetSpringDampingRatio( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_IsLimitEnabled( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_GetLowerLimit( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_GetUpperLimit( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_IsMotorEnabled( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_GetMotorSpeed( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_GetMaxMotorForce( p ) );
	b2s_put( out, capacity, n, b2PrismaticJoint_GetMotorForce( p ) );
	b2JointId r = j[4];
	b2s_put( out, capacity, n, b2RevoluteJoint_GetSpringHertz( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_GetSpringDampingRatio( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_GetAngle( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_IsLimitEnabled( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_GetLowerLimit( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_GetUpperLimit( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_IsMotorEnabled( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_GetMotorSpeed( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_GetMotorTorque( r ) );
	b2s_put( out, capacity, n, b2RevoluteJoint_GetMaxMotorTorque( r ) );
	b2JointId w = j[5];
	b2s_put( out, capacity, n, b2WeldJoint_GetLinearHertz( w ) );
	b2s_put( out, capacity, n, b2WeldJoint_GetLinearDampingRatio( w ) );
	b2s_put( out, capacity, n, b2WeldJoint_GetAngularHertz( w ) );
	b2s_put( out, capacity, n, b2WeldJoint_GetAngularDampingRatio( w ) );
	b2JointId h = j[6];
	b2s_put( out, capacity, n, b2WheelJoint_IsSpringEnabled( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_GetSpringHertz( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_GetSpringDampingRatio( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_IsLimitEnabled( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_GetLowerLimit( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_GetUpperLimit( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_IsMotorEnabled( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_GetMotorSpeed( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_GetMaxMotorTorque( h ) );
	b2s_put( out, capacity, n, b2WheelJoint_GetMotorTorque( h ) );
}

int b2s_joint_api_script( float* out, int capacity )
{
	int n = 0;
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return -1;
	b2BodyDef gd = b2DefaultBodyDef();
	b2BodyId ground = b2CreateBody( worldId, &gd );
	b2ShapeDef sd = b2DefaultShapeDef();
	b2Polygon floor = b2MakeOffsetBox( 30.0f, 0.5f, ( b2Vec2 ){ 0.0f, -0.5f }, 0.0f );
	b2CreatePolygonShape( ground, &sd, &floor );

	/* seven bodies in a row, each on its own joint to the ground or to its neighbour */
	b2BodyId body[8];
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2Polygon box = b2MakeBox( 0.4f, 0.3f );
	for ( int k = 0; k < 8; ++k )
	{
		bd.position = ( b2Vec2 ){ -10.0f + 3.0f * k, 1.0f + 0.5f * ( k & 1 ) };
		body[k] = b2CreateBody( worldId, &bd );
		b2CreatePolygonShape( body[k], &sd, &box );
	}
	b2JointId j[7];
	b2DistanceJointDef dj = b2DefaultDistanceJointDef();
	dj.bodyIdA = ground;
	dj.bodyIdB = body[0];
	dj.localAnchorA = ( b2Vec2 ){ -10.0f, 4.0f };
	dj.localAnchorB = ( b2Vec2 ){ 0.2f, 0.1f };
	dj.length = 2.5f;
	dj.enableSpring = true;
	dj.hertz = 2.0f;
	dj.dampingRatio = 0.3f;
	dj.enableLimit = true;
	dj.minLength = 2.0f;
	dj.maxLength = 3.0f;
	j[0] = b2CreateDistanceJoint( worldId, &dj );
	b2MotorJointDef mj = b2DefaultMotorJointDef();
	mj.bodyIdA = body[0];
	mj.bodyIdB = body[1];
	mj.linearOffset = ( b2Vec2 ){ 3.0f, 0.5f };
	mj.angularOffset = 0.3f;
	mj.maxForce = 100.0f;
	mj.maxTorque = 20.0f;
	mj.correctionFactor = 1.5f;
	j[1] = b2CreateMotorJoint( worldId, &mj );
	b2MouseJointDef oj = b2DefaultMouseJointDef();
	oj.bodyIdA = ground;
	oj.bodyIdB = body[2];
	oj.target = ( b2Vec2 ){ -3.5f, 3.0f };
	oj.maxForce = 50.0f;
	j[2] = b2CreateMouseJoint( worldId, &oj );
	b2PrismaticJointDef pj = b2DefaultPrismaticJointDef();
	pj.bodyIdA = ground;
	pj.bodyIdB = body[3];
	pj.localAnchorA = ( b2Vec2 ){ -1.0f, 1.5f };
	pj.localAxisA = ( b2Vec2 ){ 1.0f, 2.0f };
	pj.enableLimit = true;
	pj.lowerTranslation = 1.0f;
	pj.upperTranslation = -0.5f;
	pj.enableMotor = true;
	pj.maxMotorForce = 80.0f;
	pj.motorSpeed = 0.7f;
	j[3] = b2CreatePrismaticJoint( worldId, &pj );
	b2RevoluteJointDef rj = b2DefaultRevoluteJointDef();
	rj.bodyIdA = body[3];
	rj.bodyIdB = body[4];
	rj.localAnchorA = ( b2Vec2 ){ 1.5f, 0.25f };
	rj.localAnchorB = ( b2Vec2 ){ -1.5f, 0.0f };
	rj.referenceAngle = 4.0f;
	rj.enableLimit = true;
	rj.lowerAngle = 0.5f;
	rj.upperAngle = -0.5f;
	rj.enableSpring = true;
	rj.hertz = 1.5f;
	rj.dampingRatio = 0.2f;
	j[4] = b2CreateRevoluteJoint( worldId, &rj );
	b2WeldJointDef wj = b2DefaultWeldJointDef();
	wj.bodyIdA = body[4];
	wj.bodyIdB = body[5];
	wj.localAnchorA = ( b2Vec2 ){ 1.5f, -0.25f };
	wj.localAnchorB = ( b2Vec2 ){ -1.5f, 0.0f };
	wj.angularHertz = 2.0f;
	wj.angularDampingRatio = 0.1f;
	j[5] = b2CreateWeldJoint( worldId, &wj );
	b2WheelJointDef hj = b2DefaultWheelJointDef();
	hj.bodyIdA = body[6];
	hj.bodyIdB = body[7];
	hj.localAnchorA = ( b2Vec2 ){ 1.5f, -0.25f };
	hj.localAnchorB = ( b2Vec2 ){ -1.5f, 0.0f };
	hj.localAxisA = ( b2Vec2 ){ 0.0f, 3.0f };
	hj.enableMotor = true;
	hj.maxMotorTorque = 5.0f;
	hj.motorSpeed = 2.0f;
	hj.collideConnected = true;
	j[6] = b2CreateWheelJoint( worldId, &hj );

	b2s_joint_readout( j, out, capacity, &n );
	for ( int s = 0; s < 30; ++s )
		b2World_Step( worldId, 1.0f / 60.0f, 4 );
	b2s_joint_readout( j, out, capacity, &n );

	/* setters, including those that reset accumulated impulses */
	b2DistanceJoint_SetLength( j[0], 0.001f );
	b2DistanceJoint_SetLengthRange( j[0], 3.5f, 1.5f );
	b2DistanceJoint_EnableMotor( j[0], true );
	b2DistanceJoint_SetMotorSpeed( j[0], -0.4f );
	b2DistanceJoint_SetMaxMotorForce( j[0], 30.0f );
	b2DistanceJoint_SetSpringHertz( j[0], 3.0f );
	b2DistanceJoint_SetSpringDampingRatio( j[0], 0.6f );
	b2MotorJoint_SetLinearOffset( j[1], ( b2Vec2 ){ 2.5f, 1.0f } );
	b2MotorJoint_SetAngularOffset( j[1], 5.0f );
	b2MotorJoint_SetMaxForce( j[1], -3.0f );
	b2MotorJoint_SetMaxForce( j[1], 150.0f );
	b2MotorJoint_SetMaxTorque( j[1], 25.0f );
	b2MotorJoint_SetCorrectionFactor( j[1], 0.6f );
	b2MouseJoint_SetTarget( j[2], ( b2Vec2 ){ -2.0f, 4.0f } );
	b2MouseJoint_SetSpringHertz( j[2], 6.0f );
	b2MouseJoint_SetSpringDampingRatio( j[2], 0.9f );
	b2MouseJoint_SetMaxForce( j[2], 70.0f );
	b2PrismaticJoint_EnableSpring( j[3], true );
	b2PrismaticJoint_SetSpringHertz( j[3], 2.5f );
	b2PrismaticJoint_SetSpringDampingRatio( j[3], 0.4f );
	b2PrismaticJoint_SetLimits( j[3], 2.0f, -1.0f );
	b2PrismaticJoint_EnableMotor( j[3], false );
	b2PrismaticJoint_SetMotorSpeed( j[3], -1.0f );
	b2PrismaticJoint_SetMaxMotorForce( j[3], 60.0f );
	b2RevoluteJoint_EnableSpring( j[4], false );
	b2RevoluteJoint_SetSpringHertz( j[4], 2.0f );
	b2RevoluteJoint_SetSpringDampingRatio( j[4], 0.5f );
	b2RevoluteJoint_SetLimits( j[4], -4.0f, 4.0f );
	b2RevoluteJoint_EnableMotor( j[4], true );
	b2RevoluteJoint_SetMotorSpeed( j[4], 1.0f );
	b2RevoluteJoint_SetMaxMotorTorque( j[4], 12.0f );
	b2WeldJoint_SetLinearHertz( j[5], 4.0f );
	b2WeldJoint_SetLinearDampingRatio( j[5], 0.7f );
	b2WeldJoint_SetAngularHertz( j[5], 0.0f );
	b2WeldJoint_SetAngularDampingRatio( j[5], 0.3f );
	b2WheelJoint_EnableSpring( j[6], false );
	b2WheelJoint_SetSpringHertz( j[6], 3.0f );
	b2WheelJoint_SetSpringDampingRatio( j[6], 0.2f );
	b2WheelJoint_EnableLimit( j[6], true );
	b2WheelJoint_SetLimits( j[6], 0.3f, -0.3f );
	b2WheelJoint_SetMotorSpeed( j[6], -2.0f );
	b2WheelJoint_SetMaxMotorTorque( j[6], 8.0f );
	b2Joint_SetCollideConnected( j[6], false );
	b2Joint_SetCollideConnected( j[1], true );
	b2s_joint_readout( j, out, capacity, &n );
	for ( int s = 0; s < 30; ++s )
		b2World_Step( worldId, 1.0f / 60.0f, 4 );
	b2s_joint_readout( j, out, capacity, &n );

	/* disabling and re-enabling, and destroying a joint mid-run */
	b2DistanceJoint_EnableLimit( j[0], false );
	b2DistanceJoint_EnableSpring( j[0], false );
	b2PrismaticJoint_EnableLimit( j[3], false );
	b2RevoluteJoint_EnableLimit( j[4], false );
	b2WheelJoint_EnableMotor( j[6], false );
	b2Joint_SetCollideConnected( j[1], false );
	b2DestroyJoint( j[5] );
	for ( int s = 0; s < 30; ++s )
		b2World_Step( worldId, 1.0f / 60.0f, 4 );
	for ( int k = 0; k < 8; ++k )
	{
		b2s_put_vec( out, capacity, &n, b2Body_GetPosition( body[k] ) );
		b2Rot q = b2Body_GetRotation( body[k] );
		b2s_put( out, capacity, &n, q.c );
		b2s_put( out, capacity, &n, q.s );
	}
	b2s_put( out, capacity, &n, b2Joint_IsValid( j[5] ) ? 1.0f : 0.0f );
	b2s_put( out, capacity, &n, (float)b2Body_GetJointCount( body[4] ) );
	b2DestroyWorld( worldId );
	return n;
}

b2WorldId b2s_chain_scene( int count, uint64_t seed )
{
	b2WorldDef wd = b2s_world_def();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;
	b2sRandom rng;
	b2s_seed( &rng, seed );
	b2BodyDef gd = b2DefaultBodyDef();
	b2BodyId groundId = b2CreateBody( worldId, &gd );

	/* terrain: an open chain listed right to left, so its upper side collides */
	enum
	{
		TERRAIN = 81
	};
	b2Vec2 terrain[TERRAIN];
	float y = 0.0f;
	for ( int i = 0; i < TERRAIN; ++i )
	{
		float dy = b2s_uniform( &rng, -0.35f, 0.35f );
		y = y + dy;
		y = y < -1.0f ? -1.0f : ( y > 2.0f ? 2.0f : y );
		terrain[i] = ( b2Vec2 ){ 40.0f - 1.0f * i, y };
	}
	/* raised walls at both ends */
	terrain[0].y = 12.0f;
	terrain[TERRAIN - 1].y = 12.0f;
	b2ChainDef cd = b2DefaultChainDef();
	cd.points = terrain;
	cd.count = TERRAIN;
	cd.friction = 0.7f;
	b2CreateChain( groundId, &cd );

	/* bowl: a clockwise loop (its inside collides), open at the top by an inner lip */
	enum
	{
		HALF = 12
	};
	b2Vec2 bowl[2 * HALF];
	for ( int k = 0; k < HALF; ++k )
	{
		b2Vec2 u = b2s_circle_point( -1.0f + 2.0f * k / HALF );
		bowl[k] = ( b2Vec2 ){ -15.0f + 5.0f * u.x, 14.0f + 4.0f * u.y };
		bowl[HALF + k] = ( b2Vec2 ){ -15.0f - 5.0f * u.x, 14.0f - 4.0f * u.y };
	}
	b2Vec2 bowlCw[2 * HALF];
	for ( int k = 0; k < 2 * HALF; ++k )
		bowlCw[k] = bowl[2 * HALF - 1 - k];
	b2ChainDef bd2 = b2DefaultChainDef();
	bd2.points = bowlCw;
	bd2.count = 2 * HALF;
	bd2.isLoop = true;
	bd2.restitution = 0.2f;
	b2CreateChain( groundId, &bd2 );

	/* bodies dropped over the terrain and into the bowl */
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2ShapeDef sd = b2DefaultShapeDef();
	b2Polygon box = b2MakeBox( 0.3f, 0.2f );
	b2Polygon rounded = b2MakeRoundedBox( 0.2f, 0.2f, 0.1f );
	b2Circle circle = { { 0.0f, 0.0f }, 0.25f };
	b2Capsule capsule = { { -0.3f, 0.0f }, { 0.3f, 0.0f }, 0.15f };
	for ( int k = 0; k < count; ++k )
	{
		float px, py;
		if ( k % 8 == 7 )
		{
			/* inside the bowl */
			px = -15.0f + b2s_uniform( &rng, -2.5f, 2.5f );
			py = 13.0f + b2s_uniform( &rng, -1.0f, 2.0f );
		}
		else
		{
			px = b2s_uniform( &rng, -36.0f, 36.0f );
			py = b2s_uniform( &rng, 3.0f, 10.0f );
		}
		bd.position = ( b2Vec2 ){ px, py };
		b2BodyId id = b2CreateBody( worldId, &bd );
		switch ( k & 3 )
		{
			case 0:
				b2CreatePolygonShape( id, &sd, &box );
				break;
			case 1:
				b2CreateCircleShape( id, &sd, &circle );
				break;
			case 2:
				b2CreateCapsuleShape( id, &sd, &capsule );
				break;
			default:
				b2CreatePolygonShape( id, &sd, &rounded );
				break;
		}
	}

	/* fast bodies and bullets shot down at the terrain */
	b2Polygon pellet = b2MakeBox( 0.1f, 0.1f );
	b2Circle shot = { { 0.0f, 0.0f }, 0.1f };
	for ( int k = 0; k < 6; ++k )
	{
		bd.position = ( b2Vec2 ){ -25.0f + 10.0f * k, 8.0f };
		bd.linearVelocity = ( b2Vec2 ){ 10.0f * ( ( k & 1 ) ? 1.0f : -1.0f ), -90.0f };
		bd.isBullet = ( k % 3 ) == 0;
		b2BodyId id = b2CreateBody( worldId, &bd );
		if ( k & 1 )
			b2CreateCircleShape( id, &sd, &shot );
		else
			b2CreatePolygonShape( id, &sd, &pellet );
	}
	return worldId;
}

/* ------------------------------------------------------------ sleep scene */
static struct
{
	b2BodyId pileA[15];
	b2BodyId pileB[10];
	b2ShapeId pileBCap;
	b2BodyId links[5];
	b2JointId linkJoints[5];
	b2BodyId hover[2];
	b2BodyId slider;
	int seedDrops;
} s_sleep;

static void b2s_sleep_pile( b2WorldId worldId, b2BodyId* out, int rows, float x0 )
{
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	sd.friction = 0.6f;
	b2Polygon box = b2MakeSquare( 0.5f );
	int n = 0;
	for ( int i = 0; i < rows; ++i )
	{
		for ( int j = i; j < rows; ++j )
		{
			float x = x0 + ( i + 1.0f ) * 0.5f + ( j - i ) * 1.0f;
			float y = ( 2.0f * i + 1.0f ) * 0.5f;
			bd.position = ( b2Vec2 ){ x, y };
			out[n] = b2CreateBody( worldId, &bd );
			b2CreatePolygonShape( out[n], &sd, &box );
			n += 1;
		}
	}
}

b2WorldId b2s_sleep_scene( void )
{
	b2WorldDef wd = b2DefaultWorldDef();
	b2WorldId worldId = b2CreateWorld( &wd );
	if ( B2_IS_NULL( worldId ) )
		return worldId;
	memset( &s_sleep, 0, sizeof( s_sleep ) );

	b2BodyDef gd = b2DefaultBodyDef();
	gd.position = ( b2Vec2 ){ 0.0f, -0.5f };
	b2BodyId groundId = b2CreateBody( worldId, &gd );
	b2ShapeDef gsd = b2DefaultShapeDef();
	b2Polygon groundBox = b2MakeBox( 60.0f, 0.5f );
	b2CreatePolygonShape( groundId, &gsd, &groundBox );

	/* two resting piles: each settles into one island and falls asleep */
	b2s_sleep_pile( worldId, s_sleep.pileA, 5, -22.0f );
	b2s_sleep_pile( worldId, s_sleep.pileB, 4, -8.0f );
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	b2Circle cap = { { 0.0f, 0.6f }, 0.2f };
	s_sleep.pileBCap = b2CreateCircleShape( s_sleep.pileB[9], &sd, &cap );

	/* a damped revolute chain hanging from a static pin */
	b2BodyDef pd = b2DefaultBodyDef();
	pd.position = ( b2Vec2 ){ 5.0f, 9.0f };
	b2BodyId pinId = b2CreateBody( worldId, &pd );
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.linearDamping = 0.6f;
	bd.angularDamping = 0.6f;
	b2Capsule link = { { -0.5f, 0.0f }, { 0.5f, 0.0f }, 0.125f };
	b2BodyId prev = pinId;
	for ( int k = 0; k < 5; ++k )
	{
		bd.position = ( b2Vec2 ){ 5.5f + 1.0f * k, 9.0f };
		s_sleep.links[k] = b2CreateBody( worldId, &bd );
		b2CreateCapsuleShape( s_sleep.links[k], &sd, &link );
		b2RevoluteJointDef jd = b2DefaultRevoluteJointDef();
		jd.bodyIdA = prev;
		jd.bodyIdB = s_sleep.links[k];
		jd.localAnchorA = k == 0 ? ( b2Vec2 ){ 0.0f, 0.0f } : ( b2Vec2 ){ 0.5f, 0.0f };
		jd.localAnchorB = ( b2Vec2 ){ -0.5f, 0.0f };
		s_sleep.linkJoints[k] = b2CreateRevoluteJoint( worldId, &jd );
		prev = s_sleep.links[k];
	}

	/* two boxes created asleep in mid-air, each in a sleeping set of its own */
	b2BodyDef hd = b2DefaultBodyDef();
	hd.type = b2_dynamicBody;
	hd.isAwake = false;
	b2Polygon hoverBox = b2MakeBox( 0.75f, 0.25f );
	for ( int k = 0; k < 2; ++k )
	{
		hd.position = ( b2Vec2 ){ 14.0f + 2.5f * k, 4.0f };
		s_sleep.hover[k] = b2CreateBody( worldId, &hd );
		b2CreatePolygonShape( s_sleep.hover[k], &sd, &hoverBox );
	}

	/* a box sliding on a slippery patch */
	b2BodyDef sdef = b2DefaultBodyDef();
	sdef.type = b2_dynamicBody;
	sdef.position = ( b2Vec2 ){ 26.0f, 0.5f };
	sdef.linearVelocity = ( b2Vec2 ){ -2.0f, 0.0f };
	s_sleep.slider = b2CreateBody( worldId, &sdef );
	b2ShapeDef slick = b2DefaultShapeDef();
	slick.friction = 0.02f;
	b2Polygon sliderBox = b2MakeSquare( 0.5f );
	b2CreatePolygonShape( s_sleep.slider, &slick, &sliderBox );

	/* a kinematic platform carrying a box: its island never sleeps */
	b2BodyDef kd = b2DefaultBodyDef();
	kd.type = b2_kinematicBody;
	kd.position = ( b2Vec2 ){ 36.0f, 1.0f };
	kd.linearVelocity = ( b2Vec2 ){ 0.3f, 0.0f };
	b2BodyId platform = b2CreateBody( worldId, &kd );
	b2Polygon plate = b2MakeBox( 2.0f, 0.25f );
	b2CreatePolygonShape( platform, &sd, &plate );
	bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	bd.position = ( b2Vec2 ){ 36.0f, 1.75f };
	b2BodyId rider = b2CreateBody( worldId, &bd );
	b2CreatePolygonShape( rider, &sd, &sliderBox );
	return worldId;
}

void b2s_sleep_step( b2WorldId worldId, int step )
{
	b2ShapeDef sd = b2DefaultShapeDef();
	sd.density = 1.0f;
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	if ( step == 5 )
	{
		/* a joint between two sleeping sets merges them */
		b2DistanceJointDef dj = b2DefaultDistanceJointDef();
		dj.bodyIdA = s_sleep.hover[0];
		dj.bodyIdB = s_sleep.hover[1];
		dj.localAnchorA = ( b2Vec2 ){ 0.75f, 0.0f };
		dj.localAnchorB = ( b2Vec2 ){ -0.75f, 0.0f };
		dj.length = 1.0f;
		b2CreateDistanceJoint( worldId, &dj );
	}
	else if ( step == 60 )
	{
		/* put the sliding box's island to sleep mid-slide */
		b2Body_SetAwake( s_sleep.slider, false );
	}
	else if ( step == 120 )
	{
		/* destroying a body of the sleeping pile wakes it; its island must split later */
		b2DestroyBody( s_sleep.pileA[7] );
	}
	else if ( step == 130 )
	{
		/* removing a joint from the middle of the chain */
		b2DestroyJoint( s_sleep.linkJoints[2] );
	}
	else if ( step == 150 )
	{
		/* a box dropped onto the merged sleeping pair wakes both */
		bd.position = ( b2Vec2 ){ 14.0f, 7.0f };
		b2BodyId id = b2CreateBody( worldId, &bd );
		b2Polygon box = b2MakeSquare( 0.4f );
		b2CreatePolygonShape( id, &sd, &box );
	}
	else if ( step == 180 )
	{
		b2Body_SetAwake( s_sleep.slider, true );
	}
	else if ( step == 200 )
	{
		/* a ball rolled into the sleeping second pile */
		bd.position = ( b2Vec2 ){ -15.0f, 0.5f };
		bd.linearVelocity = ( b2Vec2 ){ 12.0f, 0.0f };
		b2BodyId id = b2CreateBody( worldId, &bd );
		b2Circle ball = { { 0.0f, 0.0f }, 0.5f };
		b2CreateCircleShape( id, &sd, &ball );
	}
	else if ( step == 220 )
	{
		b2DestroyShape( s_sleep.pileBCap );
	}
	else if ( step == 240 )
	{
		/* a velocity set on a sleeping body wakes it first */
		b2Body_SetLinearVelocity( s_sleep.slider, ( b2Vec2 ){ 1.0f, 0.0f } );
		b2Joint_WakeBodies( s_sleep.linkJoints[4] );
	}
	else if ( step == 260 )
	{
		b2Body_EnableSleep( s_sleep.pileA[0], false );
	}
	else if ( step == 290 )
	{
		b2World_EnableSleeping( worldId, false );
	}
	else if ( step == 300 )
	{
		b2World_EnableSleeping( worldId, true );
		b2Body_EnableSleep( s_sleep.pileA[0], true );
	}
}
