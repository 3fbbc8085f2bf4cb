/*
 * box2d/base.h -- export macros and process-wide hooks of the C API.
 *
 * Same public surface as the reference `include/box2d/base.h:9-107` (export macro
 * B2_API, allocator and assert hooks, version query).  Declarations are restated so a
 * C caller compiled against the reference headers links against this library unchanged.
 */
#pragma once

#include <stdint.h>

#if defined( _MSC_VER ) && defined( box2d_EXPORTS )
	#define BOX2D_EXPORT __declspec( dllexport )
#elif defined( _MSC_VER ) && defined( BOX2D_DLL )
	#define BOX2D_EXPORT __declspec( dllimport )
#elif defined( box2d_EXPORTS )
	#define BOX2D_EXPORT __attribute__( ( visibility( "default" ) ) )
#else
	#define BOX2D_EXPORT
#endif

#ifdef __cplusplus
	#define B2_API extern "C" BOX2D_EXPORT
	#define B2_INLINE inline
	#define B2_LITERAL( T ) T
	#define B2_ZERO_INIT {}
#else
	#define B2_API BOX2D_EXPORT
	#define B2_INLINE static inline
	#define B2_LITERAL( T ) ( T )
	#define B2_ZERO_INIT { 0 }
#endif

/* Host allocation hook (reference base.h:45-53).  Device memory is never routed through it. */
typedef void* b2AllocFcn( unsigned int size, int alignment );
typedef void b2FreeFcn( void* mem );

/* Assertion hook (reference base.h:56-60).  Returning non-zero requests a break. */
typedef int b2AssertFcn( const char* condition, const char* fileName, int lineNumber );

B2_API void b2SetAllocator( b2AllocFcn* allocFcn, b2FreeFcn* freeFcn );
B2_API int b2GetByteCount( void );
B2_API void b2SetAssertFcn( b2AssertFcn* assertFcn );

typedef struct b2Version
{
	int major;
	int minor;
	int revision;
} b2Version;

B2_API b2Version b2GetVersion( void );
