/*
 * error.c -- ErrorStatus construction and Python-style tracebacks.
 *
 * Behaviour follows the reference (src/error.c:25-289): errors are returned
 * by value, the traceback string is heap-owned by the caller, and every
 * WRAP_TRACEBACK frame prepends "File ..., line ... in ..." plus the call's
 * source text.  Messages are coloured with the same ANSI escapes.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "error.h"

#define C_RESET "\033[0m"
#define C_BRIGHT_RED "\033[1;31m"
#define C_DIM_RED "\033[5;31m"
#define C_YELLOW_BOLD "\033[1;33m"
#define C_CYAN "\033[0;36m"
#define C_PURPLE "\033[0;35m"
#define C_PURPLE_BOLD "\033[1;95m"

ErrorStatus make_success_error_status(void)
{
    ErrorStatus s;
    s.return_code = SUCCESS;
    s.traceback = NULL;
    s.traceback_code_ = TRACEBACK_NOT_INITIALIZED;
    return s;
}

void raise_warning(
    const char *__restrict warning_msg,
    const char *__restrict warning_file,
    const int warning_line,
    const char *__restrict warning_func
)
{
    fprintf(stderr, "%sWarning:%s In %s\"%s\"%s, line %s%d%s in %s%s%s:\n    %s%s%s\n",
            C_YELLOW_BOLD, C_RESET, C_CYAN, warning_file, C_RESET, C_CYAN, warning_line, C_RESET,
            C_CYAN, warning_func, C_RESET, C_PURPLE, warning_msg, C_RESET);
}

static const char *error_type_name(int code, int *normalized)
{
    *normalized = code;
    switch (code)
    {
        case FAILURE: return "Failure";
        case VALUE_ERROR: return "ValueError";
        case POINTER_ERROR: return "PointerError";
        case MEMORY_ERROR: return "MemoryError";
        case OS_ERROR: return "OSError";
        case NOT_IMPLEMENTED_ERROR: return "NotImplementedError";
        default:
            *normalized = UNKNOWN_ERROR;
            return "UnknownError";
    }
}

/* snprintf into a fresh buffer of exactly the needed size. */
static int format_alloc(char **out, const char *fmt, ...) __attribute__((format(printf, 2, 3)));

#include <stdarg.h>
static int format_alloc(char **out, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    const int need = vsnprintf(NULL, 0, fmt, ap);
    va_end(ap);
    *out = NULL;
    if (need < 0) return TRACEBACK_SNPRINTF_FAILED;
    char *buf = malloc((size_t) need + 1);
    if (!buf) return TRACEBACK_MALLOC_FAILED;
    va_start(ap, fmt);
    const int got = vsnprintf(buf, (size_t) need + 1, fmt, ap);
    va_end(ap);
    if (got < 0)
    {
        free(buf);
        return TRACEBACK_SNPRINTF_FAILED;
    }
    *out = buf;
    return (got > need) ? TRACEBACK_TRUNCATED : TRACEBACK_SUCCESS;
}

ErrorStatus raise_error(
    const int error_code,
    const char *__restrict error_msg,
    const char *__restrict error_file,
    const int error_line,
    const char *__restrict error_func
)
{
    ErrorStatus s;
    const char *type = error_type_name(error_code, &s.return_code);
    s.traceback = NULL;
    s.traceback_code_ = format_alloc(
        &s.traceback,
        "    File %s\"%s\"%s, line %s%d%s in %s%s%s\n%s%s%s: %s%s%s\n",
        C_CYAN, error_file, C_RESET, C_CYAN, error_line, C_RESET, C_CYAN, error_func, C_RESET,
        C_PURPLE_BOLD, type, C_RESET, C_PURPLE, error_msg, C_RESET);
    return s;
}

ErrorStatus traceback(
    ErrorStatus error_status,
    const char *__restrict function_call_source_code,
    const char *__restrict error_file,
    const int error_line,
    const char *__restrict error_func
)
{
    if (error_status.return_code == SUCCESS || error_status.traceback_code_ != TRACEBACK_SUCCESS)
    {
        return error_status;
    }
    char *frame = NULL;
    const int rc = format_alloc(
        &frame, "    File %s\"%s\"%s, line %s%d%s in %s%s%s\n        %s%s%s\n%s",
        C_CYAN, error_file, C_RESET, C_CYAN, error_line, C_RESET, C_CYAN, error_func, C_RESET,
        C_PURPLE, function_call_source_code, C_RESET, error_status.traceback);
    if (rc == TRACEBACK_MALLOC_FAILED || rc == TRACEBACK_SNPRINTF_FAILED)
    {
        free(frame);
        free(error_status.traceback);
        error_status.traceback = NULL;
        error_status.traceback_code_ = rc;
        return error_status;
    }
    free(error_status.traceback);
    error_status.traceback = frame;
    error_status.traceback_code_ = rc;
    return error_status;
}

void free_traceback(ErrorStatus *__restrict error_status)
{
    if (error_status->traceback)
    {
        free(error_status->traceback);
        error_status->traceback = NULL;
    }
}

void print_and_free_traceback(ErrorStatus *__restrict error_status)
{
    fprintf(stderr, "\n%sTraceback%s %s(most recent call last):%s\n", C_BRIGHT_RED, C_RESET, C_DIM_RED, C_RESET);
    switch (error_status->traceback_code_)
    {
        case TRACEBACK_NOT_INITIALIZED:
            fputs("    Something went wrong. Traceback not initialized.\n", stderr);
            break;
        case TRACEBACK_SUCCESS:
            fputs(error_status->traceback, stderr);
            break;
        case TRACEBACK_MALLOC_FAILED:
            fputs("    Something went wrong. Failed to allocate memory for traceback.\n", stderr);
            break;
        case TRACEBACK_TRUNCATED:
            if (error_status->traceback) fputs(error_status->traceback, stderr);
            fputs("\n    Something went wrong. Traceback are truncated.\n", stderr);
            break;
        case TRACEBACK_SNPRINTF_FAILED:
            fputs("    Something went wrong. Failed to write to traceback.\n", stderr);
            break;
        default:
            break;
    }
    free_traceback(error_status);
}
