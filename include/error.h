/*
 * error.h -- error codes and traceback helpers (reference: src/error.h).
 */
#ifndef ERROR_H
#define ERROR_H

#include "common.h"

#ifdef __cplusplus
extern "C" {
#endif

#define UNKNOWN_ERROR -1
#define SUCCESS 0
#define FAILURE 1
#define VALUE_ERROR 2
#define POINTER_ERROR 3
#define MEMORY_ERROR 4
#define OS_ERROR 5
#define NOT_IMPLEMENTED_ERROR 6

#define TRACEBACK_NOT_INITIALIZED -1
#define TRACEBACK_SUCCESS 0
#define TRACEBACK_MALLOC_FAILED 1
#define TRACEBACK_TRUNCATED 2
#define TRACEBACK_SNPRINTF_FAILED 3

#define WRAP_RAISE_WARNING(error_msg) \
    raise_warning(error_msg, __FILE__, __LINE__, __func__)

#define WRAP_RAISE_ERROR(error_code, error_msg) \
    raise_error(error_code, error_msg, __FILE__, __LINE__, __func__)

#define WRAP_TRACEBACK(function_call) \
    traceback(function_call, #function_call, __FILE__, __LINE__, __func__)

/* src/error.c:25-33 */
ErrorStatus make_success_error_status(void);

/* Print a warning to stderr (src/error.c:35-60). */
void raise_warning(
    const char *__restrict warning_msg,
    const char *__restrict warning_file,
    const int warning_line,
    const char *__restrict warning_func
);

/* Build an error status with a one-frame traceback (src/error.c:62-171). */
ErrorStatus raise_error(
    const int error_code,
    const char *__restrict error_msg,
    const char *__restrict error_file,
    const int error_line,
    const char *__restrict error_func
);

/* Prepend a frame to a failing status' traceback (src/error.c:173-252). */
ErrorStatus traceback(
    ErrorStatus error_status,
    const char *__restrict function_call_source_code,
    const char *__restrict error_file,
    const int error_line,
    const char *__restrict error_func
);

void free_traceback(ErrorStatus *__restrict error_status);
void print_and_free_traceback(ErrorStatus *__restrict error_status);

#ifdef __cplusplus
}
#endif

#endif
