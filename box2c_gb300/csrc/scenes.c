/*
 * scenes.c -- seeded synthetic scene generators (see scenes.h).
 *
 * Scene layouts follow the reference benchmark and test scenes cited per function; the
 * sizes and distributions are the ones of the five benchmark workloads (small pyramid,
 * large pyramid with x jitter, tumbler with mixed shapes, batched uneven pyramids, box
 * drops with random velocity and friction).
 */
#include "scenes.h"

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
		bd.position = ( b2Vec2 ){ cx + b2s_uniform( &rng, -slack, slack ), cy + b2s_uniform( &rng, -slack, slack ) };
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
	for ( int k = 0; k < count; ++k )
	{
		bd.position = ( b2Vec2 ){ 1.5f * k, heights[k] };
		bd.linearVelocity = ( b2Vec2 ){ vx[k], vy[k] };
		b2BodyId bodyId = b2CreateBody( worldId, &bd );
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
