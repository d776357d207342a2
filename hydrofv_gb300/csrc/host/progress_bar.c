/*
 * progress_bar.c -- a small terminal progress bar (the reference's
 * src/progress_bar.c draws a richer one; this keeps the API and prints
 * percentage, elapsed time and a linear ETA to stderr).
 */
#include <stdio.h>

#include "hydro.h"
#include "progress_bar.h"

ErrorStatus start_progress_bar(ProgressBarParam *__restrict p, const double total)
{
    p->start = hydro_get_current_time();
    p->time_last_update = p->start;
    for (int k = 0; k < 5; k++)
    {
        p->diff_time_last_five_update[k] = 0.0;
        p->last_five_progress_percent[k] = 0.0;
    }
    p->at_least_five_count = 0;
    p->current_progress = 0.0;
    p->total = total;
    return make_success_error_status();
}

void update_progress_bar(ProgressBarParam *__restrict p, double current, bool is_end)
{
    const double now = hydro_get_current_time();
    if (!is_end && now - p->time_last_update < 0.1) return;
    p->time_last_update = now;
    double frac = (p->total > 0.0) ? current / p->total : 1.0;
    if (frac > 1.0) frac = 1.0;
    if (frac < 0.0) frac = 0.0;
    p->current_progress = frac;
    const double elapsed = now - p->start;
    const double eta = (frac > 0.0) ? elapsed * (1.0 - frac) / frac : 0.0;
    const int width = 40;
    const int filled = (int) (frac * width);
    fprintf(stderr, "\r[");
    for (int k = 0; k < width; k++) fputc(k < filled ? '#' : '-', stderr);
    fprintf(stderr, "] %5.1f%%  %.1fs elapsed  ETA %.1fs", 100.0 * frac, elapsed, eta);
    if (is_end) fputc('\n', stderr);
    fflush(stderr);
}
