{
  "targets": [
    {
      "target_name": "avbd_gb300",
      "sources": ["avbd_addon.cc"],
      "include_dirs": ["<(module_root_dir)/../../include"],
      "libraries": ["-L<(module_root_dir)/../avbd_gb300", "-lavbd_gb300", "-Wl,-rpath,<(module_root_dir)/../avbd_gb300"],
      "cflags_cc": ["-std=c++17", "-O2"]
    }
  ]
}
