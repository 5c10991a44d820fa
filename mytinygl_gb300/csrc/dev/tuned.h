// tuned.h — batch defaults chosen by mytinygl_gb300/autotune.py on a GB300 (the full sweep
// is in mytinygl_gb300/tuned.json). Regenerate with that script; do not edit by hand.
#pragma once
#define MTGL_TUNED_TILE_SIZE 16
#define MTGL_TUNED_CTAS_PER_SM 8
#define MTGL_TUNED_ORDER_BY_COST 0
#define MTGL_TUNED_RECORD_FACTOR 0.47f
#define MTGL_TUNED_PAIR_FACTOR 5.8f
