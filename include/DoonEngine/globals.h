/*
 * globals.h -- core integer vector types, message callback and allocation
 * hooks of the DoonEngine API (same names, layouts and meaning as the
 * reference's src/DoonEngine/globals.h:11-81).
 */
#ifndef DN_GLOBALS_H
#define DN_GLOBALS_H

#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct DNivec2 { int32_t x, y; } DNivec2;
typedef struct DNivec3 { int32_t x, y, z; } DNivec3;
typedef struct DNivec4 { int32_t x, y, z, w; } DNivec4;
typedef struct DNuvec2 { uint32_t x, y; } DNuvec2;
typedef struct DNuvec3 { uint32_t x, y, z; } DNuvec3;
typedef struct DNuvec4 { uint32_t x, y, z, w; } DNuvec4;

/* message types and severities (globals.h:45-60) */
typedef enum DNmessageType
{
	DN_MESSAGE_CPU_MEMORY,
	DN_MESSAGE_GPU_MEMORY,
	DN_MESSAGE_SHADER,     /* kept for source compatibility; the CUDA path reports kernel launch errors here */
	DN_MESSAGE_FILE_IO
} DNmessageType;

typedef enum DNmessageSeverity
{
	DN_MESSAGE_NOTE,
	DN_MESSAGE_ERROR,
	DN_MESSAGE_FATAL
} DNmessageSeverity;

/* The message callback (globals.h:63).  The application sets it; unlike the
 * reference, the library checks for NULL before calling it. */
extern void (*g_DN_message_callback)(DNmessageType, DNmessageSeverity, const char*);

/* Host allocation used by the library.  The reference binds these at compile
 * time (globals.h:69-81); here they default to malloc/free/realloc and can
 * also be replaced at run time with DN_set_allocator (used by the
 * allocation-failure tests). */
typedef void* (*DNmallocFn)(size_t);
typedef void (*DNfreeFn)(void*);
typedef void* (*DNreallocFn)(void*, size_t);
void DN_set_allocator(DNmallocFn m, DNfreeFn f, DNreallocFn r);
void* DN_host_malloc(size_t s);
void DN_host_free(void* p);
void* DN_host_realloc(void* p, size_t s);

#ifndef DN_MALLOC
#define DN_MALLOC(s) DN_host_malloc((s))
#endif
#ifndef DN_FREE
#define DN_FREE(p) DN_host_free((p))
#endif
#ifndef DN_REALLOC
#define DN_REALLOC(p, s) DN_host_realloc((p), (s))
#endif

#ifdef __cplusplus
}
#endif

#endif
