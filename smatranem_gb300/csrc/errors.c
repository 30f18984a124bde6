/* Thread-local last-error message behind smat_last_error(). */
#include "smatran_fdtd.h"
#include "host_internal.h"

#include <stdarg.h>
#include <stdio.h>

static _Thread_local char g_msg[512];

int smat_fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    return code;
}

void smat_clear_error(void) { g_msg[0] = '\0'; }

const char *smat_last_error(void) { return g_msg; }
