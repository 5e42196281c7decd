/**
 * Device.cpp -- process-wide contexts and status-to-exception mapping.
 */
#include "Device.h"

#include <cstdlib>
#include <map>
#include <mutex>

namespace demon_gb300 {

namespace {
struct Contexts {
    std::mutex lock;
    std::map<int, dm_ctx *> byDevice;
    ~Contexts() {
        for (auto &kv : byDevice) dm_ctx_destroy(kv.second);
    }
};
Contexts &contexts() {
    static Contexts c;
    return c;
}
}  // namespace

dm_ctx *context(int device) {
    if (device < 0) {
        const char *env = std::getenv("DEMON_GB300_DEVICE");
        device = env ? std::atoi(env) : 0;
    }
    Contexts &c = contexts();
    std::lock_guard<std::mutex> g(c.lock);
    auto it = c.byDevice.find(device);
    if (it != c.byDevice.end()) return it->second;
    dm_ctx *ctx = nullptr;
    const int rc = dm_ctx_create(device, &ctx);
    if (rc != DM_OK) {
        char msg[512];
        dm_last_error(nullptr, msg, sizeof msg);
        throw Error(rc, std::string("dm_ctx_create: ") + msg);
    }
    c.byDevice[device] = ctx;
    return ctx;
}

void check(int rc, dm_ctx *ctx, const char *call) {
    if (rc == DM_OK) return;
    char msg[512] = {0};
    dm_last_error(ctx, msg, sizeof msg);
    throw Error(rc, std::string(call) + ": " + msg);
}

}  // namespace demon_gb300
