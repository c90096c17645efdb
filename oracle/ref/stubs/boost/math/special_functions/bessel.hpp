/* Test-only stub: included by a reference header, unused on the path. */
