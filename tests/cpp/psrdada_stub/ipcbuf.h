/* Declaration-only stand-in for psrdada's ipcbuf.h (psrdada is not installed
 * here): the functions and types ring.hpp's HAVE_PSRDADA clients call, with
 * the signatures of psrdada's public C API, so that code can be compiled
 * (-fsyntax-only) without the library. */
#pragma once
#include <stdint.h>
typedef struct ipcbuf_t ipcbuf_t;
char* ipcbuf_get_next_read(ipcbuf_t* id, uint64_t* bytes);
int ipcbuf_mark_cleared(ipcbuf_t* id);
char* ipcbuf_get_next_write(ipcbuf_t* id);
int ipcbuf_mark_filled(ipcbuf_t* id, uint64_t nbytes);
int ipcbuf_eod(ipcbuf_t* id);
uint64_t ipcbuf_get_bufsz(ipcbuf_t* id);
