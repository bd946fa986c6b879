{
  "targets": [
    {
      "target_name": "bcmc_node",
      "sources": ["bcmc_node.cc"],
      "include_dirs": ["../../include"],
      "cflags_cc": ["-std=c++17"],
      "libraries": ["-L<!(echo ${BCMC_LIB_DIR:-../_build})", "-lbcmc_gb300",
                    "-Wl,-rpath,<!(echo ${BCMC_LIB_DIR:-../_build})"]
    }
  ]
}
