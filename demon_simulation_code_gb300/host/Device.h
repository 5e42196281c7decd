/**
 * Device.h -- the GPU side of the host classes: one CUDA context per device
 * for the process, and C++ errors for the C ABI's status codes.
 *
 * The reference reports failures by exit(1) after a message
 * (driver.cpp:202-213); these classes throw demon_gb300::Error instead, so
 * an embedding program decides what to do.
 */
#ifndef DEMON_GB300_DEVICE_H
#define DEMON_GB300_DEVICE_H

#include <stdexcept>
#include <string>

#include "demon_gb300.h"

namespace demon_gb300 {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string &what) : std::runtime_error(what), status(status) {}
    const int status;  //!< dm_status of the failing call
};

/// The process-wide context of CUDA device `device` (created on first use;
/// device -1 = $DEMON_GB300_DEVICE, default 0).
dm_ctx *context(int device = -1);

/// Throws Error with the context's last message if rc != DM_OK.
void check(int rc, dm_ctx *ctx, const char *call);

}  // namespace demon_gb300

#endif  // DEMON_GB300_DEVICE_H
