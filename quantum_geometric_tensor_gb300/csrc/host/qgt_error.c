/*
 * qgt_error.c -- thread-local last-error text.  The reference keeps one static
 * string (src/quantum_geometric/core/quantum_geometric_tensor_network.c:16-24),
 * which is not thread-safe; here every thread has its own.
 */
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "../qgt_internal.h"

static _Thread_local char g_msg[512];
static _Thread_local int g_code;

int qgt_set_error(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    g_code = code;
    return code;
}

void qgt_clear_error(void)
{
    g_msg[0] = 0;
    g_code = 0;
}

const char* qgt_last_error(void) { return g_msg[0] ? g_msg : "No error"; }

const char* qgt_version(void) { return "qgt-gb300 0.1 (sm_103a)"; }
