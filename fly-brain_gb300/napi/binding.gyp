{
  "targets": [
    {
      "target_name": "flybrain_napi",
      "sources": ["flybrain_napi.c"],
      "include_dirs": ["../../include"],
      "libraries": ["-L<(module_root_dir)/../flybrain/_lib", "-lflybrain", "-Wl,-rpath,<(module_root_dir)/../flybrain/_lib"],
      "cflags": ["-O2", "-std=c11"]
    }
  ]
}
