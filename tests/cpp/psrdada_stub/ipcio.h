/* Declaration-only stand-in for psrdada's ipcio.h (see ipcbuf.h). */
#pragma once
#include <sys/types.h>
#include "ipcbuf.h"
typedef struct ipcio_t ipcio_t;
char* ipcio_open_block_read(ipcio_t* ipc, uint64_t* curbufsz, uint64_t* block_id);
ssize_t ipcio_close_block_read(ipcio_t* ipc, uint64_t bytes);
char* ipcio_open_block_write(ipcio_t* ipc, uint64_t* block_id);
ssize_t ipcio_close_block_write(ipcio_t* ipc, uint64_t bytes);
