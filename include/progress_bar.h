/*
 * progress_bar.h -- terminal progress bar (reference: src/progress_bar.h).
 */
#ifndef PROGRESS_BAR_H
#define PROGRESS_BAR_H

#include <time.h>

#include "common.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ProgressBarParam
{
    double start;
    double time_last_update;
    double diff_time_last_five_update[5];
    double last_five_progress_percent[5];
    int at_least_five_count;
    double current_progress;
    double total;
} ProgressBarParam;

ErrorStatus start_progress_bar(ProgressBarParam *__restrict progress_bar_param, const double total);
void update_progress_bar(ProgressBarParam *__restrict progress_bar_param, double current, bool is_end);

#ifdef __cplusplus
}
#endif

#endif
