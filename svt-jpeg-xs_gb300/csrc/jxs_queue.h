/*
 * Ordered frame-slot queue shared by the encoder and decoder handles.
 *
 * Replaces the reference's thread/FIFO runtime for this path
 * (Source/Lib/Common/Codec/Threads/SystemResourceManager.c:361-660 and the
 * final-stage reorder ring, Encoder/Codec/FinalStageProcess.c:89-263): a
 * frame takes a GPU slot at send time, results are handed out strictly in
 * submission order, and one library thread waits for completions so that
 * the "data available" callbacks fire from a single thread, one at a time.
 */
#ifndef JXS_QUEUE_H
#define JXS_QUEUE_H

#include <pthread.h>
#include <stdint.h>

#define JXS_Q_MAX 8

enum { SLOT_FREE = 0, SLOT_ACQUIRED = 1, SLOT_SUBMITTED = 2, SLOT_DONE = 3 };

typedef int32_t (*jxs_wait_fn)(void* ctx, int slot);
typedef void (*jxs_cb_fn)(void* ctx);

typedef struct jxs_queue {
    int nslots;
    int state[JXS_Q_MAX];
    int32_t err[JXS_Q_MAX];
    int on_gpu[JXS_Q_MAX];       /* slot has GPU work to wait for */
    int order[JXS_Q_MAX];
    int head, count;
    int stop;
    int pending_send_cb;
    pthread_mutex_t mu;
    pthread_cond_t cv;
    pthread_t th;
    int th_started;
    jxs_wait_fn wait_fn;
    jxs_cb_fn get_cb, send_cb;
    void* ctx;
} jxs_queue_t;

int jxs_queue_init(jxs_queue_t* q, int nslots, jxs_wait_fn wait_fn, jxs_cb_fn get_cb, jxs_cb_fn send_cb, void* ctx);
void jxs_queue_shutdown(jxs_queue_t* q);
/* Takes a free slot (appended to the output order).  Returns -1 when none is
 * free and blocking is 0. */
int jxs_queue_acquire(jxs_queue_t* q, int blocking);
/* The slot's work is queued on the GPU (on_gpu) or already final (err). */
void jxs_queue_submitted(jxs_queue_t* q, int slot, int on_gpu, int32_t err);
/* Oldest slot once it is done; -1 if not done and blocking is 0. */
int jxs_queue_peek_done(jxs_queue_t* q, int blocking, int32_t* err);
/* Releases the oldest slot. */
void jxs_queue_pop(jxs_queue_t* q);

#endif
