// Host-side types shared by the model builder and the C ABI.
#pragma once
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "mx_model.h"

namespace mx {

struct Pack {
  struct Section { int dtype; size_t count; std::vector<char> data; };
  std::map<std::string, Section> sections;
  bool load(const char *path, std::string &err);
  template <class T> const T *get(const std::string &name, size_t *count, std::string &err) const;
};

// Host copies of every device table, plus the scalar launch parameters.
struct HostModel {
  MxTables T;
  std::vector<MxShellDev> shells;
  std::vector<float> optc;
  std::vector<double> optc_slope;
  std::vector<double> fold_hdr, fold_ealpha, fold_inv_de;
  std::vector<float> fold_theta;
  std::vector<MxGratingDev> gratings;
  std::vector<float> geff_energy, geff_cum;
  std::vector<double> order_k, sectors;
  std::vector<MxChipDev> chips;
  std::vector<float> support_energy, support_cum;
  std::vector<double> support_k;
  std::vector<float> hrc_tab;
  std::vector<double> hrc_slope;
  std::vector<int32_t> fef_map;
  std::vector<MxFefDev> fef;
  std::vector<float> fef_f;
  std::vector<double> fef_slope;
  std::vector<MxContamDev> contam;
};

bool build_model(const Pack &pk, const mx_config &cfg, HostModel &M, std::string &err);

}  // namespace mx
