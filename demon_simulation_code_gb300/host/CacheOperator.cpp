/**
 * CacheOperator.cpp -- host substep inputs; the products and sums are
 * separate roundings (0.5 * l, then + x), as in the reference's SSE build.
 */
#include "CacheOperator.h"

void CacheOperator::operation1(const double currentTime) { (void)currentTime; }

namespace {
void half_step(Cloud *c, const double *l, const double *nn, const double *k, const double *m) {
    for (cloud_index i = 0; i < c->n; i++) {
        c->xCache[i] = 0.5 * l[i] + c->x[i];
        c->yCache[i] = 0.5 * nn[i] + c->y[i];
        c->VxCache[i] = 0.5 * k[i] + c->Vx[i];
        c->VyCache[i] = 0.5 * m[i] + c->Vy[i];
    }
}
}  // namespace

void CacheOperator::operation2(const double currentTime) {
    (void)currentTime;
    half_step(cloud, cloud->l1, cloud->n1, cloud->k1, cloud->m1);
}

void CacheOperator::operation3(const double currentTime) {
    (void)currentTime;
    half_step(cloud, cloud->l2, cloud->n2, cloud->k2, cloud->m2);
}

void CacheOperator::operation4(const double currentTime) {
    (void)currentTime;
    for (cloud_index i = 0; i < cloud->n; i++) {
        cloud->xCache[i] = cloud->x[i] + cloud->l3[i];
        cloud->yCache[i] = cloud->y[i] + cloud->n3[i];
        cloud->VxCache[i] = cloud->Vx[i] + cloud->k3[i];
        cloud->VyCache[i] = cloud->Vy[i] + cloud->m3[i];
    }
}
