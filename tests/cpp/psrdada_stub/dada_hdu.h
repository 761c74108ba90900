/* Declaration-only stand-in for psrdada's dada_hdu.h (see ipcbuf.h). */
#pragma once
#include <sys/types.h>
#include "ipcbuf.h"
#include "ipcio.h"
typedef struct multilog_t multilog_t;
typedef struct dada_hdu {
  multilog_t* log;
  ipcio_t* data_block;
  ipcbuf_t* header_block;
} dada_hdu_t;
dada_hdu_t* dada_hdu_create(multilog_t* log);
void dada_hdu_set_key(dada_hdu_t* hdu, key_t key);
int dada_hdu_connect(dada_hdu_t* hdu);
int dada_hdu_disconnect(dada_hdu_t* hdu);
void dada_hdu_destroy(dada_hdu_t* hdu);
int dada_hdu_lock_read(dada_hdu_t* hdu);
int dada_hdu_unlock_read(dada_hdu_t* hdu);
int dada_hdu_lock_write(dada_hdu_t* hdu);
int dada_hdu_unlock_write(dada_hdu_t* hdu);
