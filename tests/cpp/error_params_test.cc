// The host-side error bounds of the C++ mirror (RnsErrorParams in
// rlwe_gpu.h), which need no GPU: prints, for the parameters on the command
// line (log_n log_t sigma max_log_b num_digits q...), B_plaintext,
// B_secretkey_encryption, B_publickey_encryption, B_scale and
// BoundOnGadgetBasedKeySwitching(1, max_log_b, num_digits) as %.17g, one per
// line, or the status message of a rejected parameter set.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rlwe_gpu.h"

int main(int argc, char** argv) {
  if (argc < 7) return 2;
  const int log_n = std::atoi(argv[1]), log_t = std::atoi(argv[2]);
  const double sigma = std::atof(argv[3]);
  const int log_b = std::atoi(argv[4]), digits = std::atoi(argv[5]);
  std::vector<uint64_t> qs;
  for (int i = 6; i < argc; ++i) qs.push_back(std::strtoull(argv[i], nullptr, 10));
  if (qs.size() == 1 && qs[0] == 0) qs.clear();
  auto ep = rlwe_gpu::RnsErrorParams::Create(log_n, qs, {}, log_t, sigma);
  if (!ep.ok()) {
    std::printf("%s\n", std::string(ep.status().message()).c_str());
    return 1;
  }
  std::printf("%.17g\n%.17g\n%.17g\n%.17g\n%.17g\n", ep->B_plaintext(),
              ep->B_secretkey_encryption(), ep->B_publickey_encryption(), ep->B_scale(),
              ep->BoundOnGadgetBasedKeySwitching(1, log_b, digits));
  return 0;
}
