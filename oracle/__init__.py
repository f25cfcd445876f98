"""Oracle package: CPU restatement of the reference's filter path plus the
recipe that compiles the reference's own sources.  Test infrastructure only;
the product never imports it."""
