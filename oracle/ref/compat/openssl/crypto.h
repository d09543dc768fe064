// Test infrastructure: nothing of BoringSSL's crypto.h is used by the shim build.
#pragma once
