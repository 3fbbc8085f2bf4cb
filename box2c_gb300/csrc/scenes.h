/*
 * scenes.h -- seeded synthetic scene generators for the benchmark workloads.
 *
 * The generators use only the public box2d C API, so the same source is compiled
 * against this library, against the plain-C oracle and against the reference build;
 * each copy lives in its own shared object next to the backend it drives.  Random
 * numbers come from PCG32 (O'Neill 2014) and float arithmetic without transcendental
 * functions, so a seed produces bit-identical scenes on x86-64 and aarch64.
 */
#pragma once

#include "box2d/box2d.h"

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* PCG32 stream state. */
typedef struct b2sRandom
{
	uint64_t state;
	uint64_t inc;
} b2sRandom;

void b2s_seed( b2sRandom* rng, uint64_t seed );
uint32_t b2s_next( b2sRandom* rng );
/* Uniform in [lo, hi). */
float b2s_uniform( b2sRandom* rng, float lo, float hi );
/* Zero-mean unit-variance normal approximated by the Irwin-Hall sum of 12 uniforms. */
float b2s_normal( b2sRandom* rng );

/* Default world definition of every benchmark scene: sleep off, continuous on
 * (reference benchmark/main.c:185-186). */
b2WorldDef b2s_world_def( void );

/* Pyramid of unit boxes on a 200 m x 1 m static ground whose top face is y = 0.
 * Row i (0-based) holds baseCount - i boxes; each box centre gets x jitter uniform in
 * [-jitter, jitter] from `seed` (no jitter when jitter == 0).  Layout follows the
 * reference benchmark/large_pyramid.c:34-50.  Returns the world. */
b2WorldId b2s_pyramid( int baseCount, float jitter, uint64_t seed );

/* Adds the pyramid bodies to an existing world (used to pack several into one). */
void b2s_add_pyramid( b2WorldId worldId, int baseCount, float jitter, uint64_t seed, float xOffset );

/* Motor-driven hollow box (20 x 20 m, 1 m thick walls, density 50) on a revolute joint
 * to a shapeless static ground.  variant 0: `count` bodies alternating boxes of
 * half-extent 0.125 and circles of radius 0.125 at seeded jittered-grid positions
 * inside, motor 0.05*pi rad/s.  variant 1: the reference benchmark scene
 * (benchmark/tumbler.c:8-80): a 45 x 45 grid of 0.125 boxes, motor 25 deg/s. */
b2WorldId b2s_tumbler( int count, uint64_t seed, int variant );

/* `count` boxes of half-extent 0.5 at x = 1.5 k, y = heights[k], initial velocity
 * (vx[k], vy[k]), on the pyramid ground; every shape uses `friction`. */
b2WorldId b2s_drop_boxes( int count, const float* heights, const float* vx, const float* vy, float friction );
/* The same with body k's shape chosen by kinds[k]: 0 a unit box, 1 a circle of radius
 * 0.5, 2 a capsule (0.6 long, radius 0.25), 3 a plank 0.4 thick spanning the row of
 * bodies (centred under it; with more than eleven bodies on it, its contacts overflow
 * the graph colours); kinds null means boxes. */
b2WorldId b2s_drop_shapes( int count, const float* heights, const float* vx, const float* vy, float friction, const int* kinds );

/* Reference benchmark/joint_grid.c: an n x n grid of circles (radius 0.4, filtered so
 * that no two touch) with revolute joints to the neighbours above and to the left; the
 * seven centre bodies of the top row are static.  The benchmark has n = 100 and no
 * gravity; a negative gravityY makes the grid hang and swing from its static anchors. */
b2WorldId b2s_joint_grid( int n, float gravityY );

/* Reference benchmark/many_pyramids.c: rowCount x columnCount pyramids of baseCount
 * boxes (half-extent 0.5, default material), each row of pyramids standing on its own
 * static segment; sleep off.  The benchmark has 20 x 20 pyramids of base 10. */
b2WorldId b2s_many_pyramids( int rowCount, int columnCount, int baseCount );

/* Mixed-shape pile in a static funnel of segments (floor, two slopes) with a static
 * capsule bar and a static box ledge: `count` bodies dropped from a seeded jittered
 * grid, in turn a horizontal capsule, a box, a circle, a rounded box and an upright
 * capsule.  Every registered shape pair of the narrowphase occurs. */
b2WorldId b2s_shape_pile( int count, uint64_t seed );

/* Revolute joint scene: a hub circle pinned to a static anchor, `spokes` boxes on a ring
 * pinned to the hub and to each other (the hub's joints beyond the colours go to the
 * overflow set), `chains` six-link capsule chains swinging from static pins, and twelve
 * boxes dropped onto them.  flags: 1 joint limits, 2 joint springs, 4 motors. */
b2WorldId b2s_joint_hub( int spokes, int chains, int flags, uint64_t seed );

/* Contact-free revolute chains: `chains` chains of `links` capsules (filtered so that no
 * two shapes touch) swinging from static pins, with joint limits (flags & 1), damped
 * springs (flags & 2) and motors on every third joint (flags & 4). */
b2WorldId b2s_joint_chains( int chains, int links, int flags, uint64_t seed );

/* Continuous collision scene: `count` small projectiles (circles, boxes, capsules; every
 * fourth a bullet) fired at 60 to 120 m/s at a 0.1 m thick static wall, past a column of
 * ten dynamic boxes, above a static ground segment. */
b2WorldId b2s_fast_shots( int count, uint64_t seed );

/* Destruction scene: a pyramid, a hub with 14 pinned spokes (some joints in the
 * overflow set) and bodies of two shapes on a static ledge.  b2s_destruction_step,
 * called after each step with the step number, destroys pyramid bodies (step 20), spoke
 * joints (40), one shape of each two-shape body (60), the hub (80), creates bodies that
 * reuse the freed ids (100) and destroys the static ledge (120).  One such scene at a
 * time per process. */
b2WorldId b2s_destruction( void );
void b2s_destruction_step( b2WorldId worldId, int step );

/* Building blocks of the reference's test/test_world.c checks: a world of the default
 * definition (gravity, sleep on), a body of the default definition and the given type
 * at the origin, and a dynamic body at the origin with a square of half-extent h. */
b2WorldId b2s_empty_world( void );
b2BodyId b2s_add_body( b2WorldId worldId, int type );
b2BodyId b2s_add_square( b2WorldId worldId, float h );

/* Event scene: `count` boxes and circles dropped through a static sensor band onto a
 * ground whose shape reports hit events; some bodies bounce (restitution 0.6), every
 * other one enables hit events, every fifth disables contact events, every seventh
 * carries a sensor ring of radius 0.8. */
b2WorldId b2s_event_scene( int count, uint64_t seed );

/* Joint scene with every joint type: `copies` copies 40 m apart on one static ground,
 * each with a distance-joint rope (soft with length limits, rigid, motorised), a
 * revolute pendulum (spring, limits, motor), two prismatic elevators (motor and limits;
 * spring on a tilted axis), a car on two sprung wheel joints with a rear motor, a weld
 * cantilever (rigid and soft welds), a motor joint and a mouse joint to the ground, a
 * fourteen-legged spider whose hub joints of every type overflow the graph colours,
 * and twelve seeded boxes and circles dropped over them.  flags & 1: the rope and
 * elevator joints let their bodies collide. */
b2WorldId b2s_joint_zoo( int copies, int flags, uint64_t seed );

/* Chain scene: a static open chain of 80 links over seeded uneven terrain with raised
 * ends, a closed clockwise loop (a bowl whose inside collides), `count` boxes, circles,
 * capsules and rounded boxes dropped over them (every eighth into the bowl), and six
 * fast bodies (two of them bullets) shot down at the terrain. */
b2WorldId b2s_chain_scene( int count, uint64_t seed );

/* Joint API script: one joint of each type between a ground and eight boxes; reads
 * every joint query (configuration, reaction force and torque, type-specific values)
 * before and after 30 steps, calls every setter (clamping ones with out-of-range values,
 * impulse-resetting ones, collide-connected toggles), steps and reads again, then
 * disables features, destroys a joint, steps and reads the bodies.  Writes up to
 * `capacity` floats to out; returns the number written (-1 without a world). */
int b2s_joint_api_script( float* out, int capacity );

/* Sleep scene (world and bodies with sleep on): two resting piles of boxes, a damped
 * revolute chain from a static pin, two boxes created asleep in mid-air, a box sliding
 * on a slippery patch and a kinematic platform carrying a box.  b2s_sleep_step, called
 * after each step with the step number, joins the two sleeping boxes (merging their
 * sets, step 5), puts the slider to sleep (60), destroys a body of the sleeping first
 * pile (120) and a joint of the chain (130), drops a box onto the sleeping pair (150),
 * wakes the slider (180), rolls a ball into the second pile (200), destroys a shape of
 * it (220), sets the sleeping slider's velocity and wakes the chain's end (240),
 * disables one body's sleep (260) and the world's (290), and enables both again (300).
 * One such scene at a time per process. */
b2WorldId b2s_sleep_scene( void );
void b2s_sleep_step( b2WorldId worldId, int step );

/* Draws `n` integers uniform in [lo, hi] from `seed` into out. */
void b2s_draw_ints( int n, uint64_t seed, int lo, int hi, int* out );
/* Draws `n` floats uniform in [lo, hi) / standard normal from `seed` into out. */
void b2s_draw_uniform( int n, uint64_t seed, float lo, float hi, float* out );
void b2s_draw_normal( int n, uint64_t seed, float* out );

/* Reference unit-test scenes: test/test_world.c:17-97 (HelloWorld) and
 * test/test_determinism.c:87-177 (10 x 10 rounded-box tilted stacks). */
b2WorldId b2s_hello_world( b2BodyId* bodyOut );
b2WorldId b2s_tilted_stacks( void );

#ifdef __cplusplus
}
#endif
