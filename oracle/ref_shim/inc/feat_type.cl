typedef short feat_t;
