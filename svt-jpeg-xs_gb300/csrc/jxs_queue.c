#include "jxs_queue.h"

#include <string.h>

static void* completion_thread(void* arg) {
    jxs_queue_t* q = (jxs_queue_t*)arg;
    pthread_mutex_lock(&q->mu);
    if (q->send_cb) {
        /* initial room in the input queue (InitStageProcess.c:165-168) */
        pthread_mutex_unlock(&q->mu);
        q->send_cb(q->ctx);
        pthread_mutex_lock(&q->mu);
    }
    for (;;) {
        int slot = -1;
        for (int i = 0; i < q->count; i++) {
            int s = q->order[(q->head + i) % JXS_Q_MAX];
            if (q->state[s] == SLOT_ACQUIRED) break; /* keep output order */
            if (q->state[s] == SLOT_SUBMITTED) {
                slot = s;
                break;
            }
        }
        if (slot < 0) {
            if (q->pending_send_cb > 0 && q->send_cb) {
                q->pending_send_cb--;
                pthread_mutex_unlock(&q->mu);
                q->send_cb(q->ctx);
                pthread_mutex_lock(&q->mu);
                continue;
            }
            if (q->stop) break;
            pthread_cond_wait(&q->cv, &q->mu);
            continue;
        }
        int32_t err = q->err[slot];
        if (q->on_gpu[slot]) {
            pthread_mutex_unlock(&q->mu);
            int32_t e = q->wait_fn(q->ctx, slot);
            pthread_mutex_lock(&q->mu);
            if (!err) err = e;
        }
        q->err[slot] = err;
        q->state[slot] = SLOT_DONE;
        pthread_cond_broadcast(&q->cv);
        if (q->get_cb) {
            pthread_mutex_unlock(&q->mu);
            q->get_cb(q->ctx);
            pthread_mutex_lock(&q->mu);
        }
    }
    pthread_mutex_unlock(&q->mu);
    return NULL;
}

int jxs_queue_init(jxs_queue_t* q, int nslots, jxs_wait_fn wait_fn, jxs_cb_fn get_cb, jxs_cb_fn send_cb, void* ctx) {
    memset(q, 0, sizeof(*q));
    if (nslots < 1) nslots = 1;
    if (nslots > JXS_Q_MAX) nslots = JXS_Q_MAX;
    q->nslots = nslots;
    q->wait_fn = wait_fn;
    q->get_cb = get_cb;
    q->send_cb = send_cb;
    q->ctx = ctx;
    pthread_mutex_init(&q->mu, NULL);
    pthread_cond_init(&q->cv, NULL);
    if (pthread_create(&q->th, NULL, completion_thread, q) != 0) return -1;
    q->th_started = 1;
    return 0;
}

void jxs_queue_shutdown(jxs_queue_t* q) {
    if (!q->th_started) return;
    pthread_mutex_lock(&q->mu);
    q->stop = 1;
    pthread_cond_broadcast(&q->cv);
    pthread_mutex_unlock(&q->mu);
    pthread_join(q->th, NULL);
    q->th_started = 0;
    pthread_cond_destroy(&q->cv);
    pthread_mutex_destroy(&q->mu);
}

int jxs_queue_acquire(jxs_queue_t* q, int blocking) {
    pthread_mutex_lock(&q->mu);
    for (;;) {
        if (q->count < q->nslots) {
            for (int s = 0; s < q->nslots; s++) {
                if (q->state[s] == SLOT_FREE) {
                    q->state[s] = SLOT_ACQUIRED;
                    q->err[s] = 0;
                    q->on_gpu[s] = 0;
                    q->order[(q->head + q->count) % JXS_Q_MAX] = s;
                    q->count++;
                    pthread_mutex_unlock(&q->mu);
                    return s;
                }
            }
        }
        if (!blocking || q->stop) {
            pthread_mutex_unlock(&q->mu);
            return -1;
        }
        pthread_cond_wait(&q->cv, &q->mu);
    }
}

void jxs_queue_submitted(jxs_queue_t* q, int slot, int on_gpu, int32_t err) {
    pthread_mutex_lock(&q->mu);
    q->on_gpu[slot] = on_gpu;
    q->err[slot] = err;
    q->state[slot] = SLOT_SUBMITTED;
    pthread_cond_broadcast(&q->cv);
    pthread_mutex_unlock(&q->mu);
}

int jxs_queue_peek_done(jxs_queue_t* q, int blocking, int32_t* err) {
    pthread_mutex_lock(&q->mu);
    for (;;) {
        if (q->count > 0) {
            int s = q->order[q->head];
            if (q->state[s] == SLOT_DONE) {
                *err = q->err[s];
                pthread_mutex_unlock(&q->mu);
                return s;
            }
        }
        if (!blocking || (q->stop && q->count == 0)) {
            pthread_mutex_unlock(&q->mu);
            return -1;
        }
        pthread_cond_wait(&q->cv, &q->mu);
    }
}

void jxs_queue_pop(jxs_queue_t* q) {
    pthread_mutex_lock(&q->mu);
    if (q->count > 0) {
        int s = q->order[q->head];
        q->state[s] = SLOT_FREE;
        q->head = (q->head + 1) % JXS_Q_MAX;
        q->count--;
        q->pending_send_cb++;
        pthread_cond_broadcast(&q->cv);
    }
    pthread_mutex_unlock(&q->mu);
}
