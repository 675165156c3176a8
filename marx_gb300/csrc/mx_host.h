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
  double geom_area_cm2 = 0.0;   // Marx_Mirror_Geometric_Area (hrma.c:736): the open aperture area, cm^2
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

// The parameters of a MARX parameter file (name,type,mode,value,... per
// line) plus "Name=value" overrides, a later entry winning (mx_par.cpp).
struct ParSet {
  std::vector<std::pair<std::string, std::string>> kv;
  const std::string *find(const std::string &name) const;
};
bool load_par(const char *path, const char *const *overrides, int n_overrides, ParSet &out, std::string &err);
// An mx_param_reader over a ParSet (user: the ParSet).
int par_reader(void *user, const char *name, char type, char *value, size_t len);

}  // namespace mx
