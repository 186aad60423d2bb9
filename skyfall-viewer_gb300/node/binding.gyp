{
  "targets": [
    {
      "target_name": "skyfall_addon",
      "sources": ["skyfall_addon.c"],
      "include_dirs": ["../../include"],
      "libraries": [
        "-L<(module_root_dir)/../skyfall",
        "-lskyfall",
        "-Wl,-rpath,<(module_root_dir)/../skyfall"
      ],
      "cflags": ["-std=c11", "-Wall"]
    }
  ]
}
